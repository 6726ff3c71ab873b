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
#include <array>
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
    cudaFree(pos);
    cudaFree(rank_at);
    cudaFree(ublk);
    cudaFree(sched_hdr);
    cudaFree(sched_ent);
    cudaFree(sched16);
    cudaFree(up_diag_d);
    cudaFree(up_diag_f);
    cudaFree(up_imp);
    cudaFree(up4);
    cudaFree(rs);
    cudaFree(rs_row);
    cudaFree(rs_blob);
    cudaFree(blob);
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
        // Sites without couplings have no moves: they share one subsystem.
        // Beyond kMaxSub subsystems the two smallest are merged (a merged
        // count is still conserved, the blocks are only coarser).
        std::vector<int> size(nsub, 0), coupled(nsub, 0);
        for (int i = 0; i < m.nsite; ++i) size[ctx->site_subsys[i]]++;
        for (int i = 0; i < m.ncpl; ++i) coupled[ctx->site_subsys[ctx->cpl_orb[i]]] = 1;
        std::vector<int> remap(nsub, -1);
        int nnew = 0, inert = -1;
        for (int k = 0; k < nsub; ++k) {
            if (coupled[k]) {
                remap[k] = nnew++;
            } else {
                if (inert < 0) inert = nnew++;
                remap[k] = inert;
            }
        }
        for (int i = 0; i < m.nsite; ++i) ctx->site_subsys[i] = remap[ctx->site_subsys[i]];
        nsub = nnew;
        while (nsub > kMaxSub) {
            std::vector<int> sz(nsub, 0);
            for (int i = 0; i < m.nsite; ++i) sz[ctx->site_subsys[i]]++;
            int a1 = 0;
            for (int k = 1; k < nsub; ++k)
                if (sz[k] < sz[a1]) a1 = k;
            int a2 = a1 == 0 ? 1 : 0;
            for (int k = 0; k < nsub; ++k)
                if (k != a1 && sz[k] < sz[a2]) a2 = k;
            const int lo = std::min(a1, a2), hi = std::max(a1, a2);
            for (int i = 0; i < m.nsite; ++i) {
                int &v = ctx->site_subsys[i];
                if (v == hi) v = lo;
                else if (v > hi) --v;
            }
            --nsub;
        }
        ctx->nsub = nsub;
    }
    if (!ctx->d_mdl) MOED_CUDA(ctx, cudaMalloc(&ctx->d_mdl, sizeof(ModelDev)));
    MOED_CUDA(ctx, cudaMemcpyAsync(ctx->d_mdl, &m, sizeof(m), cudaMemcpyHostToDevice, ctx->stream));
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // species tables, H*v tile lists and tile-shape choices belong to the model
    ctx->hv_tiles.clear();
    ctx->hv_choice.clear();
    ctx->hv_times.clear();
    ctx->species.clear();
    return upload_binom(ctx);
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

// ---------------------------------------------------------------------------
// Species tables of the conserved-block layout, built on the host (nsite <=
// 15: at most 6435 words per species) and uploaded once.
// ---------------------------------------------------------------------------
namespace {

inline int par_below(unsigned w, int bit) { return __builtin_popcount(w & ((1u << bit) - 1u)) & 1; }

struct Hop {
    int tgt;    // target rank
    int cidx;   // coupling index: 1 + 2*coupling + negative sign
    int sub;    // subsystem the move stays in
};

// Hybridisation moves of a word in the reference's loop order (iorb outer,
// ibath inner; hybridization1 then hybridization2, ed_hamiltonian.F90:146-161).
// Signs: product of the destruction and creation signs (parity of occupied
// bits below the operated bit, ed_operators.F90:292-348).  For the down
// species the reference also counts every up-spin bit below; that parity
// appears in both operators and cancels.
void word_hops(const mo_ed_ctx *ctx, const std::vector<int> &rank, unsigned w, std::vector<Hop> &out)
{
    out.clear();
    for (size_t i = 0; i < ctx->cpl_val.size(); ++i) {
        const int o = ctx->cpl_orb[i], k = ctx->cpl_bath[i];
        const int ob = (w >> o) & 1, kb = (w >> k) & 1;
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
        const int s1 = par_below(w, src);
        const unsigned w1 = w & ~(1u << src);
        const int s2 = par_below(w1, dst);
        const unsigned w2 = w1 | (1u << dst);
        out.push_back({rank[w2], 1 + 2 * (int)i + ((s1 ^ s2) & 1), ctx->site_subsys[o]});
    }
}

// Impurity transfer T_{i<-j} (c+_i c_j on one species): valid when j is
// occupied and i empty; sign from the two operators' parities.
bool transfer(unsigned w, int i, int j, unsigned *w2, int *neg)
{
    if (!((w >> j) & 1) || ((w >> i) & 1)) return false;
    const int s1 = par_below(w, j);
    const unsigned w1 = w & ~(1u << j);
    const int s2 = par_below(w1, i);
    *w2 = w1 | (1u << i);
    *neg = (s1 ^ s2) & 1;
    return true;
}

template <typename T>
int upload_vec(mo_ed_ctx *ctx, T **dst, const std::vector<T> &src)
{
    cudaFree(*dst);
    *dst = nullptr;
    MOED_CUDA(ctx, cudaMalloc(dst, sizeof(T) * std::max<size_t>(1, src.size())));
    if (!src.empty())
        MOED_CUDA(ctx, cudaMemcpyAsync(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice,
                                       ctx->stream));
    return MO_ED_OK;
}

}  // namespace

int get_species(mo_ed_ctx *ctx, int N, Species **out)
{
    auto it = ctx->species.find(N);
    if (it != ctx->species.end()) {
        *out = it->second.get();
        return MO_ED_OK;
    }
    const int nsite = ctx->nsite, nsub = ctx->nsub, norb = ctx->norb;
    const ModelDev &m = ctx->mdl;
    std::unique_ptr<Species> s(new Species);
    s->nsite = nsite;
    s->N = N;
    s->n = (int)binom(nsite, N);
    s->nsub = nsub;
    const int n = s->n;

    // words in ascending order (the reference's basis order) and their ranks
    std::vector<int> rank(1u << nsite, -1);
    s->h_words.reserve(n);
    for (unsigned w = 0; w < (1u << nsite); ++w)
        if (__builtin_popcount(w) == N) {
            rank[w] = (int)s->h_words.size();
            s->h_words.push_back((int)w);
        }

    // subsystem masks; local state index of every sub-pattern (ascending
    // within each subsystem and electron count)
    unsigned smask[kMaxSub] = {0};
    for (int i = 0; i < nsite; ++i) smask[ctx->site_subsys[i]] |= 1u << i;
    std::vector<int> lidx(1u << nsite, 0);
    for (int k = 0; k < nsub; ++k) {
        int cnt[kMaxSite + 2] = {0};
        unsigned sub = 0;
        while (true) {   // submasks of smask[k] in ascending order
            lidx[sub] = cnt[__builtin_popcount(sub)]++;
            if (sub == smask[k]) break;
            sub = (sub - smask[k]) & smask[k];
        }
    }
    auto counts_of = [&](unsigned w, int *c) {
        for (int k = 0; k < nsub; ++k) c[k] = __builtin_popcount(w & smask[k]);
    };

    // blocks: distinct count tuples, lexicographic
    std::map<std::vector<int>, int> bkey;
    for (int r = 0; r < n; ++r) {
        int c[kMaxSub];
        counts_of((unsigned)s->h_words[r], c);
        bkey.emplace(std::vector<int>(c, c + nsub), 0);
    }
    const int nblk = (int)bkey.size();
    std::vector<std::vector<int>> bcnt;
    std::vector<std::array<int, kMaxSub>> bL(nblk), bstride(nblk);
    {
        int b = 0;
        for (auto &kv : bkey) {
            kv.second = b++;
            bcnt.push_back(kv.first);
        }
    }
    s->h_ublk.resize(nblk);
    s->h_ublk_cnt.assign((size_t)nblk * kMaxSub, 0);
    int col = 0;
    for (int b = 0; b < nblk; ++b) {
        int W = 1;
        for (int k = nsub - 1; k >= 0; --k) {
            bL[b][k] = (int)binom(__builtin_popcount(smask[k]), bcnt[b][k]);
            bstride[b][k] = W;
            W *= bL[b][k];
            s->h_ublk_cnt[(size_t)b * kMaxSub + k] = bcnt[b][k];
        }
        UpBlock &u = s->h_ublk[b];
        u.col0 = col;
        u.W = W;
        u.W4 = (W + 3) & ~3;
        u.hdr0 = 0;
        u.s16_off = u.s16_bytes = u.pad0 = u.pad1 = 0;
        col += u.W4;
    }
    s->ncol = col;
    s->ld = std::max(32, (col + 31) & ~31);
    if (s->ld > 65535) return fail(ctx, MO_ED_ERR_ARG, "species too wide for the 16-bit column tables");
    const int ld = s->ld;
    std::vector<int> blk_of(n), idx_of(n);
    s->h_pos.assign(n, 0);
    s->h_rank_at.assign(ld, -1);
    for (int r = 0; r < n; ++r) {
        const unsigned w = (unsigned)s->h_words[r];
        int c[kMaxSub];
        counts_of(w, c);
        const int b = bkey.at(std::vector<int>(c, c + nsub));
        int idx = 0;
        for (int k = 0; k < nsub; ++k) idx += lidx[w & smask[k]] * bstride[b][k];
        blk_of[r] = b;
        idx_of[r] = idx;
        s->h_pos[r] = s->h_ublk[b].col0 + idx;
        s->h_rank_at[s->h_pos[r]] = r;
    }

    // per word: moves, diagonal, impurity pattern
    std::vector<std::vector<Hop>> hops(n);
    std::vector<double> diag(n);
    for (int r = 0; r < n; ++r) {
        const unsigned w = (unsigned)s->h_words[r];
        word_hops(ctx, rank, w, hops[r]);
        // onsite (ed_operators.F90:68-84) + same-spin (U-3J) n_i n_j over
        // impurity orbitals (dens_dens, ed_operators.F90:157-159)
        double d = 0.0;
        for (int i = 0; i < nsite; ++i)
            if ((w >> i) & 1) d += ctx->ek[i];
        for (int i = 0; i < norb; ++i)
            for (int j = i + 1; j < norb; ++j)
                if (((w >> i) & 1) && ((w >> j) & 1)) d += ctx->U - 3 * ctx->J;
        diag[r] = d;
    }
    const bool four = ctx->J != 0.0 && m.npair > 0;
    int pidx[kMaxOrb][kMaxOrb] = {{0}};
    {
        int p = 0;
        for (int i = 0; i < norb; ++i)
            for (int j = 0; j < norb; ++j)
                if (i != j) pidx[i][j] = p++;
    }

    // ---- up-spin role: per-column tables and gather schedules ----
    std::vector<double> updd(ld, 0.0);
    std::vector<float> updf(ld, 0.0f);
    std::vector<unsigned char> upimp(ld, 0);
    std::vector<unsigned> up4((size_t)std::max(1, m.npair) * ld, 0u);
    for (int r = 0; r < n; ++r) {
        const int c = s->h_pos[r];
        const unsigned w = (unsigned)s->h_words[r];
        updd[c] = diag[r];
        updf[c] = (float)diag[r];
        upimp[c] = (unsigned char)(w & (unsigned)(m.nimp - 1));
        if (!four) continue;
        for (int i = 0; i < norb; ++i)
            for (int j = 0; j < norb; ++j) {
                if (i == j) continue;
                unsigned w2;
                int neg;
                if (transfer(w, i, j, &w2, &neg))
                    up4[(size_t)pidx[i][j] * ld + c] =
                        0x80000000u | ((unsigned)neg << 30) | (unsigned)s->h_pos[rank[w2]];
            }
    }
    std::vector<int2> hdr;
    std::vector<unsigned> ent;
    for (int b = 0; b < nblk; ++b) {
        UpBlock &u = s->h_ublk[b];
        const int nq = u.W4 / 4, nch = (nq + 15) / 16;
        u.hdr0 = (int)hdr.size();
        for (int ch = 0; ch < nch; ++ch)
            for (int k = 0; k < 4; ++k) {
                // lanes: the 16 columns 4*l + k of the chunk; banks: target mod 32 (the
                // two half-warps read two rows, which may then meet in a bank)
                std::vector<int> el, eb, et, ec;
                int ldeg[16] = {0}, bdeg[32] = {0};
                for (int l = 0; l < 16; ++l) {
                    const int c = 4 * (16 * ch + l) + k;
                    if (c >= u.W) continue;
                    const int r = s->h_rank_at[u.col0 + c];
                    for (const Hop &h : hops[r]) {
                        const int tc = s->h_pos[h.tgt] - u.col0;
                        if (tc < 0 || tc >= u.W) return fail(ctx, MO_ED_ERR_ARG, "up-spin move leaves its block");
                        el.push_back(l);
                        eb.push_back(tc & 31);
                        et.push_back(tc);
                        ec.push_back(h.cidx);
                        ldeg[l]++;
                        bdeg[tc & 31]++;
                    }
                }
                int delta = 0;
                for (int t = 0; t < 16; ++t) delta = std::max(delta, ldeg[t]);
                for (int t = 0; t < 32; ++t) delta = std::max(delta, bdeg[t]);
                std::vector<int> colour;
                if (!el.empty()) colour_chunk(el, eb, delta, colour);
                const int first = (int)ent.size();
                ent.resize(ent.size() + (size_t)16 * delta, 0xffffffffu);
                std::vector<unsigned> used((size_t)delta, 0u);
                for (size_t e = 0; e < el.size(); ++e) {
                    ent[first + 16 * colour[e] + el[e]] = (unsigned)et[e] | ((unsigned)ec[e] << 16);
                    used[colour[e]] |= 1u << eb[e];
                }
                for (int sl = 0; sl < delta; ++sl)
                    for (int l = 0; l < 16; ++l) {
                        unsigned &x = ent[first + 16 * sl + l];
                        if (x != 0xffffffffu) continue;
                        // no move: read a bank no other lane of the slot uses
                        int t = -1;
                        for (int bb = 0; bb < 32 && bb < u.W4; ++bb)
                            if (!((used[sl] >> bb) & 1u)) {
                                t = bb;
                                used[sl] |= 1u << bb;
                                break;
                            }
                        if (t < 0) t = std::min(4 * (16 * ch + l) + k, u.W4 - 1);
                        x = (unsigned)t;
                    }
                hdr.push_back(make_int2(first, delta));
                s->sched_slots_max = std::max(s->sched_slots_max, delta);
            }
    }

    // 16-bit copies of the block schedules (staged into shared memory by the
    // H*v kernel) where every target and coupling index fits
    std::vector<unsigned char> s16;
    for (int b = 0; b < nblk; ++b) {
        UpBlock &u = s->h_ublk[b];
        const int nh = (u.W4 / 4 + 15) / 16 * 4;
        if (u.W4 > 1024 || 2 * m.ncpl + 1 > 64) continue;
        const int e0 = hdr[u.hdr0].x;
        const int e1 = hdr[u.hdr0 + nh - 1].x + 16 * hdr[u.hdr0 + nh - 1].y;
        const size_t bytes = ((size_t)4 * nh + 2 * (size_t)(e1 - e0) + 15) & ~(size_t)15;
        std::vector<unsigned char> bl(bytes, 0);
        for (int h = 0; h < nh; ++h) {
            const unsigned w = ((unsigned)(hdr[u.hdr0 + h].x - e0) << 8) | (unsigned)hdr[u.hdr0 + h].y;
            memcpy(&bl[4 * h], &w, 4);
        }
        for (int e = e0; e < e1; ++e) {
            const unsigned x = ent[e];
            const unsigned short v = (unsigned short)((x & 0xffffu) | ((x >> 16) << 10));
            memcpy(&bl[4 * nh + 2 * (size_t)(e - e0)], &v, 2);
        }
        u.s16_off = (int)(s16.size() / 16);
        u.s16_bytes = (int)bytes;
        s16.insert(s16.end(), bl.begin(), bl.end());
    }

    // ---- down-spin role: row sets at every level, with their metadata blobs ----
    s->h_dblk.assign(nblk, DownBlock());
    std::vector<std::vector<int>> members(nblk);
    for (int r = 0; r < n; ++r) members[blk_of[r]].push_back(r);
    std::vector<int2> rsv, rblob;
    std::vector<int> rrow;
    std::vector<unsigned char> blob;
    auto a16 = [](size_t v) { return (v + 15) & ~(size_t)15; };
    for (int b = 0; b < nblk; ++b) {
        DownBlock &db = s->h_dblk[b];
        db.size = (int)members[b].size();
        for (int k = 0; k < nsub; ++k) db.cnt[k] = bcnt[b][k];
        // row axis order: subsystems with fewer moves first, so that the
        // trailing (closed) axes carry the most moves
        std::vector<double> mv(nsub, 0.0);
        for (int r : members[b])
            for (const Hop &h : hops[r]) mv[h.sub] += 1.0;
        std::vector<int> ax(nsub);
        for (int k = 0; k < nsub; ++k) ax[k] = k;
        std::stable_sort(ax.begin(), ax.end(), [&](int x, int y) { return mv[x] < mv[y]; });
        std::vector<int> inpos(nsub);
        for (int t = 0; t < nsub; ++t) inpos[ax[t]] = t;
        for (int j = 0; j <= nsub; ++j) {
            int nset = 1, rows = 1;
            for (int t = 0; t < nsub; ++t) (t < j ? nset : rows) *= bL[b][ax[t]];
            db.rs0[j] = (int)rsv.size();
            db.nset[j] = nset;
            db.rs_rows[j] = rows;
            db.blob_max[j] = 0;
            // set index / index in the set of a word of this block
            auto place = [&](unsigned w, int *set, int *row) {
                int sv = 0, rv = 0;
                for (int t = 0; t < nsub; ++t) {
                    const int li = lidx[w & smask[ax[t]]];
                    if (t < j) sv = sv * bL[b][ax[t]] + li;
                    else rv = rv * bL[b][ax[t]] + li;
                }
                *set = sv;
                *row = rv;
            };
            std::vector<int> at((size_t)nset * rows, -1);
            for (int r : members[b]) {
                int sv, rv;
                place((unsigned)s->h_words[r], &sv, &rv);
                at[(size_t)sv * rows + rv] = r;
            }
            for (int q = 0; q < nset; ++q) {
                const int rec0 = (int)rrow.size();
                rsv.push_back(make_int2(rec0, rows));
                std::vector<int4> info(rows);
                std::vector<double> dg(rows);
                std::vector<unsigned> mvs, q4s;
                for (int rv = 0; rv < rows; ++rv) {
                    const int r = at[(size_t)q * rows + rv];
                    if (r < 0) return fail(ctx, MO_ED_ERR_ARG, "row set with a missing row");
                    rrow.push_back(r);
                    const unsigned w = (unsigned)s->h_words[r];
                    dg[rv] = diag[r];
                    const int mv0 = (int)mvs.size();
                    int nin = 0, nopen = 0;
                    for (const Hop &h : hops[r])
                        if (inpos[h.sub] >= j) {
                            int s2, r2;
                            place((unsigned)s->h_words[h.tgt], &s2, &r2);
                            mvs.push_back((unsigned)r2 | ((unsigned)h.cidx << 16));
                            ++nin;
                        }
                    for (const Hop &h : hops[r])
                        if (inpos[h.sub] < j) {
                            mvs.push_back((unsigned)h.tgt | ((unsigned)h.cidx << 16));
                            ++nopen;
                        }
                    const int q0 = (int)q4s.size();
                    int n4 = 0;
                    if (four)
                        for (int i = 0; i < norb; ++i)
                            for (int jj = 0; jj < norb; ++jj) {
                                if (i == jj) continue;
                                const int p = pidx[i][jj];
                                unsigned w2;
                                int neg;
                                // spin-flip: the down spin moves i -> j (T_{j<-i})
                                if (transfer(w, jj, i, &w2, &neg)) {
                                    q4s.push_back((unsigned)rank[w2] | ((unsigned)p << 16) | ((unsigned)neg << 22));
                                    ++n4;
                                }
                                // pair hopping: the down spin moves j -> i (T_{i<-j})
                                if (transfer(w, i, jj, &w2, &neg)) {
                                    q4s.push_back((unsigned)rank[w2] | ((unsigned)p << 16) | (1u << 21) |
                                                  ((unsigned)neg << 22));
                                    ++n4;
                                }
                            }
                    info[rv] = make_int4((int)(w & (unsigned)(m.nimp - 1)) | (nin << 8) | (nopen << 16) | (n4 << 24),
                                         mv0, q0, r);
                }
                const size_t off_info = 16, off_diag = off_info + 16 * (size_t)rows;
                const size_t off_mv = a16(off_diag + 8 * (size_t)rows);
                const size_t off_q4 = a16(off_mv + 4 * mvs.size());
                const size_t total = a16(off_q4 + 4 * q4s.size());
                const size_t base = blob.size();
                blob.resize(base + total, 0);
                const int4 head = make_int4(rows, (int)off_mv, (int)off_q4, (int)total);
                memcpy(&blob[base], &head, 16);
                memcpy(&blob[base + off_info], info.data(), 16 * (size_t)rows);
                memcpy(&blob[base + off_diag], dg.data(), 8 * (size_t)rows);
                if (!mvs.empty()) memcpy(&blob[base + off_mv], mvs.data(), 4 * mvs.size());
                if (!q4s.empty()) memcpy(&blob[base + off_q4], q4s.data(), 4 * q4s.size());
                rblob.push_back(make_int2((int)(base / 16), (int)total));
                db.blob_max[j] = std::max(db.blob_max[j], (int)total);
            }
        }
    }
    s->nrs = (int)rsv.size();
    s->nrec = (int)rrow.size();

    // the device basis: combinadic unrank / rank kernels (the host lists
    // above give the same words; they only drive the table construction)
    MOED_CUDA(ctx, cudaMalloc(&s->words, sizeof(int) * std::max(1, n)));
    MOED_CUDA(ctx, cudaMalloc(&s->rank, sizeof(int) << nsite));
    {
        const int T = 256;
        k_unrank<<<(n + T - 1) / T, T, 0, ctx->stream>>>(nsite, N, n, s->words);
        MOED_CHECK_LAUNCH(ctx);
        k_rank<<<((1 << nsite) + T - 1) / T, T, 0, ctx->stream>>>(nsite, N, s->rank);
        MOED_CHECK_LAUNCH(ctx);
    }
    if (int rc = upload_vec(ctx, &s->pos, s->h_pos)) return rc;
    if (int rc = upload_vec(ctx, &s->rank_at, s->h_rank_at)) return rc;
    if (int rc = upload_vec(ctx, &s->ublk, s->h_ublk)) return rc;
    if (int rc = upload_vec(ctx, &s->sched_hdr, hdr)) return rc;
    if (int rc = upload_vec(ctx, &s->sched_ent, ent)) return rc;
    if (int rc = upload_vec(ctx, &s->up_diag_d, updd)) return rc;
    if (int rc = upload_vec(ctx, &s->up_diag_f, updf)) return rc;
    if (int rc = upload_vec(ctx, &s->up_imp, upimp)) return rc;
    if (int rc = upload_vec(ctx, &s->up4, up4)) return rc;
    if (blob.size() / 16 > (size_t)0x7fffffff) return fail(ctx, MO_ED_ERR_ARG, "row-set metadata too large");
    s->h_rs = rsv;
    s->h_rs_blob = rblob;
    if (int rc = upload_vec(ctx, &s->sched16, s16)) return rc;
    if (int rc = upload_vec(ctx, &s->rs, rsv)) return rc;
    if (int rc = upload_vec(ctx, &s->rs_row, rrow)) return rc;
    if (int rc = upload_vec(ctx, &s->rs_blob, rblob)) return rc;
    if (int rc = upload_vec(ctx, &s->blob, blob)) return rc;
    MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
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
