// internal.h -- shared declarations of the GB300 ED solver (sm_103a).
//
// Data layout in HBM
//   A sector vector X of dimension D = nup*ndown is stored on the device as
//   ndown rows of nup elements, X[idown][iup] -- the reference's row order
//   (ed_basis.F90:120-123,137-138: row index iup + (idown-1)*nup) -- with the
//   row stride padded to ld = roundup(nup, 32) so that every row starts on a
//   128-byte boundary (pad elements are zero).  Host entry points convert to
//   and from the unpadded reference layout with one 2D copy.  Every H*v term
//   that moves only up-spin electrons stays inside a row; down-spin moves are
//   whole-row AXPYs.
//
//   Per spin species (nsite sites, N electrons) the device holds
//     words[n]          ascending state words (colex unrank),
//     rank[2^nsite]     inverse table (-1 outside the species),
//     hop_tgt/val[hw][n] up to hw compacted hybridisation moves per word
//                        (slot-major so a warp reading slot s of 32
//                        consecutive words is coalesced),
//     hop_cnt[n]        number of valid moves,
//     diag[n]           species part of the diagonal.
//   Because the impurity orbitals are the lowest bits, words sharing their
//   bath bits are contiguous in rank order ("bath groups"); spin-flip and
//   pair-hopping only move within a bath group by a rank offset that depends
//   on the impurity bits alone, kept in a 2^norb-entry table.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mo_ed.h"

namespace moed {

constexpr int kMaxSite = 15;      // 2*nsite <= 30 bits in an int32 state word (ed_config.f90:8)
constexpr int kMaxOrb = 5;        // impurity orbitals handled by the 4-operator tables
constexpr int kMaxPair = kMaxOrb * (kMaxOrb - 1);
constexpr int kMaxImp = 1 << kMaxOrb;
constexpr int kMaxHop = 64;       // max nonzero couplings norb*nbath (15 sites: <= 56)

// ---------------------------------------------------------------------------
// device model constants (one per context; rebuilt by mo_ed_set_model)
// ---------------------------------------------------------------------------
struct ModelDev {
    int norb, nbath, nsite, npair, nimp, ncpl;
    double U, J;
    // 4-operator transfer table T_{i<-j}(I) for impurity pattern I and ordered
    // pair p=(i,j): bit31 valid, bit30 negative sign, low 16 bits signed rank delta
    int t4[kMaxPair * kMaxImp];
    int pair_rev[kMaxPair];       // index of (j,i) for p=(i,j)
    unsigned pairmask[kMaxImp];   // bit p set iff T_p(I) is valid
    double cval[kMaxHop];         // nonzero couplings V in the reference loop order
    double cross[kMaxImp * kMaxImp];  // interspecies diagonal U n_i^up n_i^dn + (U-2J) n_i^up n_j^dn
};

// ---------------------------------------------------------------------------
// spin species tables
// ---------------------------------------------------------------------------
template <typename T>
struct HopEnt;                    // one up-spin move of a column: target rank and signed coupling
template <>
struct alignas(8) HopEnt<float> {
    int t;
    float v;
};
template <>
struct alignas(16) HopEnt<double> {
    int t, pad;
    double v;
};

struct Species {
    int nsite = 0, N = 0, n = 0, hw = 0;
    int n_pad = 0;                // roundup(n, 32): row stride when this species is the up spin
    int *words = nullptr;
    int *rank = nullptr;
    int *hop_cnt = nullptr;
    int *hop_tgt = nullptr;       // [hw][n]
    double *hop_val_d = nullptr;  // [hw][n]
    float *hop_val_f = nullptr;
    int *info = nullptr;          // [n_pad]: hop count | impurity bits << 8 (pads: 0)
    double *diag_d = nullptr;     // [n_pad] (pads: 0)
    float *diag_f = nullptr;
    // column move tables, chunk-major: entry (chunk c = u/4, slot s, u%4) at
    // (c*hw + s)*4 + u%4, so one thread reads the slot-s moves of its four
    // columns as one contiguous 32-byte (FP32) / 64-byte (FP64) block
    HopEnt<float> *tab_f = nullptr;
    HopEnt<double> *tab_d = nullptr;
    // conflict-free gather schedule of the up-spin moves: per 32-column chunk
    // c, sched_hdr[c] = {first entry, slots}; entry (slot s, lane l) at
    // first + 32*s + l is 0 (no move) or valid | neg << 22 | coupling << 16 |
    // target rank.  Within a slot the 32 targets fall in 32 different
    // shared-memory banks (target mod 32).
    int2 *sched_hdr = nullptr;
    unsigned *sched_ent = nullptr;
    std::vector<int2> h_sched_hdr;    // host copies (per-R tables derive from them)
    std::vector<unsigned> h_sched_ent;
    int sched_slots_max = 0;
    // per rows-per-item R: the schedule as {shared-memory offset of row 0 in
    // the [tile][R][32] stage, signed coupling}; empty lanes read a bank that
    // no other lane of the slot uses, with coupling 0
    std::map<int, HopEnt<float> *> sched_rf;
    std::map<int, HopEnt<double> *> sched_rd;
    int max_cnt = 0;              // largest hop_cnt over words
    int max_group = 0;            // largest bath group (words sharing their bath bits)
    // row items for a given rows-per-item R: whole bath groups packed into
    // items of <= R rows (rank order inside a group), items sorted by the
    // bath-occupation counts of the conserved subsystems; -1 pads
    std::map<int, int *> items;   // R -> [nitems][R]
    // per-item descriptors of the staged H*v kernel, key R*2 + (FP64 ? 1 : 0)
    std::map<int, unsigned *> desc;
    std::map<int, int> nitems;
    // down-spin blocks of the split H*v: rows with equal electron counts in
    // every conserved subsystem, closed under hybridisation moves.  Positions
    // p run over the rows block by block (largest block first).
    int dblk_n = 0, dblk_max = 0, dblk_mvmax = 0;  // blocks, largest block, most moves in a block
    int *dblk_off = nullptr;      // [dblk_n + 1] first position of each block
    int *dblk_rows = nullptr;     // [n] row (rank) at position p
    int *dblk_ptr = nullptr;      // [n + 1] first move of position p
    // moves of each position: {target index within the block, signed coupling}
    HopEnt<float> *dblk_mv_f = nullptr;
    HopEnt<double> *dblk_mv_d = nullptr;
    // per row stride ld: {first chunk, 32-column units per chunk} of each block
    std::map<int, int2 *> dblk_chunks;
    std::map<int, int> dblk_nchunks;
    std::vector<int> dblk_h_off;  // host copy of dblk_off
    ~Species();
};

struct Sector {
    int ne_up, ne_down;
    Species *up, *dn;
    long long D() const { return (long long)up->n * dn->n; }     // dimension
    int ld() const { return up->n_pad; }                           // device row stride
    long long Dpad() const { return (long long)up->n_pad * dn->n; } // device elements
};

// ---------------------------------------------------------------------------
// H*v job (one vector of one sector); the kernel walks a list of jobs
// ---------------------------------------------------------------------------
template <typename TA>
struct HvJobT {
    const void *x;            // input vector (TX), device layout
    void *y;                  // output vector (TY), device layout
    double *dot_partial;      // optional [nitems]: sum over the item of x*y
    const int *active;        // optional device flag: job skipped when *active == 0
    int nu, nd, ld;
    int item0, nitems;
    const int *items;         // [nitems][R] rows of each item (-1 pads)
    const int *up_info;       // [ld]: move count | impurity bits << 8
    const HopEnt<TA> *up_tab; // chunk-major column moves
    const TA *up_diag;        // [ld]
    int up_hw, up_maxcnt;
    const int *dn_info;       // [nd]
    const int *dn_tgt;        // [hw][nd]
    const TA *dn_val;         // [hw][nd]
    const TA *dn_diag;        // [nd]
    int dn_maxcnt, pad;
    const int2 *up_sched_hdr;      // conflict-free gather schedule (Species::sched_*)
    const unsigned *up_sched_ent;
    const HopEnt<TA> *up_sched;
    const unsigned *desc;          // per-item descriptors (staged kernel)
    // down-spin blocks of the split kernel (Species::dblk_*)
    const int *dblk_off, *dblk_rows, *dblk_ptr;
    const HopEnt<TA> *dblk_mv;
    const int2 *dblk_chunks;
    int dblk_n, dblk_max, dblk_mvmax;
    int tile0, ntiles;             // this job's chunks in the batch (split kernel)
};

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct DevBuf {              // owning device allocation (move-only)
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes)
    {
        o.p = nullptr;
        o.bytes = 0;
    }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            bytes = o.bytes;
            o.p = nullptr;
            o.bytes = 0;
        }
        return *this;
    }
    void release();
    ~DevBuf() { release(); }
};

struct StateVec {             // an eigenpair kept on the device after ed_solve
    int sector;               // 0-based index into the sector list
    int level;                // 0-based level within the sector
    double val, prob;
    double pev = 0.0;         // Boltzmann factor before normalisation (eigenvalues.dat)
    int prec;                 // MO_ED_FP32 / MO_ED_FP64: the precision of vec
    DevBuf vec;               // Dpad elements in the layout of its sector
};

struct GreenRecord {          // one apbpanbn.dat record (ed_green.F90:112-115)
    int iev, iorb, even;
    double val, prob;
    int np, nn;
    std::vector<double> ap, bp, an, bn;
};

}  // namespace moed

struct mo_ed_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 0;
    std::string err;
    mo_ed_options opt;
    long long launches = 0;

    // model
    bool have_model = false;
    int norb = 0, nbath = 0, nsite = 0;
    double U = 0, J = 0;
    std::vector<double> ek, vk;   // vk column-major (norb fastest)
    moed::ModelDev mdl;
    moed::ModelDev *d_mdl = nullptr;
    std::vector<int> cpl_orb, cpl_bath;  // nonzero couplings in reference loop order
    std::vector<double> cpl_val;
    std::vector<int> site_subsys;  // conserved subsystem (orbital + coupled bath levels) of each site
    int dblk_bound = 0;            // largest down-spin block over every electron count
    int dblk_mv_bound = 0;         // most hybridisation moves in one such block
    std::map<int, std::unique_ptr<moed::Species>> species;  // by N

    // statistics of the last eigensolve (mo_ed_diag_stats)
    int diag_cycles = 0;
    long long diag_matvecs = 0;
    double diag_res_est = 0.0, diag_res_true = 0.0;
    double refine_res = 0.0;   // largest Ritz residual of the last FP64 refinement (green_fp64)
    // the last bath fit (mo_ed_fit_stats): suspensions, persistent clusters
    long long fit_suspensions = 0;
    int fit_clusters = 0;

    // sectors / omega
    std::vector<int> nelec, nup;
    std::vector<double> omega;

    // results of ed_solve / green
    std::vector<moed::StateVec> states;
    std::vector<moed::GreenRecord> green;
    // square-lattice band of the DMFT self-consistency (mo_ed_set_band_structure)
    moed::DevBuf d_hk;
    int nq = 0;

    // scratch
    moed::DevBuf scratch_a, scratch_b, scratch_part;
    // eigensolver workspace reused across sectors (Krylov vectors of sectors
    // up to 64 MB per vector, and the projected-problem arrays)
    std::vector<moed::DevBuf> trl_pool, trl_small, rr_pool;
    // autotuned H*v tile shape per (kind, Nup, Ndn), and the timings (ms) of
    // every shape measured when it was chosen (negative: did not fit)
    std::map<long long, int> hv_choice;
    std::map<long long, std::vector<float>> hv_times;
    // worker contexts of mo_ed_solve's threads (same device and model, own
    // streams and workspace), with the model generation each one holds
    std::vector<mo_ed_ctx *> workers;
    std::vector<long long> worker_gen;
    long long model_gen = 0;   // incremented by every mo_ed_set_model
};

namespace moed {

// ---- error helpers --------------------------------------------------------
int fail(mo_ed_ctx *ctx, int code, const std::string &msg);
int cuda_fail(mo_ed_ctx *ctx, cudaError_t e, const char *what);
#define MOED_CUDA(ctx, call)                                              \
    do {                                                                  \
        cudaError_t e_ = (call);                                          \
        if (e_ != cudaSuccess) return ::moed::cuda_fail((ctx), e_, #call); \
    } while (0)
#define MOED_CHECK_LAUNCH(ctx)                                            \
    do {                                                                  \
        (ctx)->launches++;                                                \
        cudaError_t e_ = cudaGetLastError();                              \
        if (e_ != cudaSuccess) return ::moed::cuda_fail((ctx), e_, "kernel launch"); \
    } while (0)

int dev_alloc(mo_ed_ctx *ctx, DevBuf &b, size_t bytes);
int ensure(mo_ed_ctx *ctx, DevBuf &b, size_t bytes);
// host vector in the reference layout (D contiguous) <-> device vector in the
// padded layout (ndown rows of stride ld, zero pads); es = element size.
int upload_padded(mo_ed_ctx *ctx, const Sector &s, const void *host, void *dev, size_t es);
int download_padded(mo_ed_ctx *ctx, const Sector &s, const void *dev, void *host, size_t es);

// ---- tables (tables.cu) ----------------------------------------------------
long long binom(int n, int k);
int build_model(mo_ed_ctx *ctx);
int get_species(mo_ed_ctx *ctx, int N, Species **out);
int get_sector(mo_ed_ctx *ctx, int ne_up, int ne_down, Sector *out);
// Lookup only: MO_ED_ERR_STATE when the sector's tables were never built
// (get_sector builds them, and allocates; this never allocates).
int find_sector(mo_ed_ctx *ctx, int ne_up, int ne_down, Sector *out);
int basis_get_dev(mo_ed_ctx *ctx, const Sector &s, long long n, const long long *d_idx,
                  unsigned *d_state);
int basis_idx_dev(mo_ed_ctx *ctx, const Sector &s, long long n, const unsigned *d_state,
                  long long *d_idx);

// ---- H*v (hv.cu) ------------------------------------------------------------
enum HvKind { HV_F64 = 0, HV_F32 = 1, HV_MIXED = 2 };
// Fill a job for sector s (x, y device pointers) with R rows per item (the
// item table for R must exist: hv_prepare / hv_prepare_rows).
template <typename TA>
void hv_fill_job(const mo_ed_ctx *ctx, const Sector &s, int R, const void *x, void *y, HvJobT<TA> &job);
// Launch H*v over a host list of jobs (item0 is assigned here); jobs are
// passed to the kernel by value, so the call can be captured in a CUDA graph.
// v = tile-shape variant (hv_prepare); all jobs use its rows per item.
int hv_launch_f32(mo_ed_ctx *ctx, int v, const HvJobT<float> *jobs, int njobs);
int hv_launch_f64(mo_ed_ctx *ctx, int kind, int v, const HvJobT<double> *jobs, int njobs);
int species_items(mo_ed_ctx *ctx, Species *sp, int R, const int **items, int *nitems);
// Tile-shape variant for sector s (autotuned on the first call per shape;
// that first call allocates and synchronizes, so make it before any stream
// capture) and its rows per item; builds the item table.
int hv_prepare(mo_ed_ctx *ctx, const Sector &s, int kind, int *v, int *R);
// autotuner record of a shape: per variant (R, NT, MINB) and time in ms
int hv_tuning(mo_ed_ctx *ctx, const Sector &s, int kind, int cap, int *nvar, int *shape, float *ms, int *chosen);
// tables of variant v (item table, schedule, descriptors) for a sector
// batched with the one v was tuned on
int hv_prepare_rows(mo_ed_ctx *ctx, const Sector &s, int kind, int v);
// Per-R stage offsets of the up-spin gather schedule (built once per R).
int species_sched(mo_ed_ctx *ctx, Species *sp, int R);
// Down-spin block tables of a species (split H*v), built once; chunk table
// for row stride ld.
int species_dblocks(mo_ed_ctx *ctx, Species *sp, int ld);
// Lookup only: the tile shape and item table that hv_prepare left for this
// sector and kind, or MO_ED_ERR_STATE if it never ran (never tunes or allocates).
int hv_lookup(mo_ed_ctx *ctx, const Sector &s, int kind, int *v, int *R);
// Pin the tile-shape variant of a sector and kind (instead of the autotuner's choice).
int hv_set_variant(mo_ed_ctx *ctx, const Sector &s, int kind, int v);
// Convenience: one vector, jobs staged through scratch.
int hv_single(mo_ed_ctx *ctx, const Sector &s, int kind, const void *x, void *y);

// ---- Krylov (krylov.cu) -----------------------------------------------------
int lanczos_reference(mo_ed_ctx *ctx, const Sector &s, const double *h_vec, int nstep,
                      int *nstep_calc, double *a, double *b);
// The same recurrence with every device buffer carved from the caller's
// region [scratch, scratch + cap) (256-byte aligned).  Needs hv_lookup to
// succeed for the sector; allocates no device memory.  Bytes needed:
size_t lanczos_region_bytes(const Sector &s, int prec, int nstep, int hv_rows);
// Look up (and so commit) the no-allocation region on the context's device.
int noalloc_prepare(mo_ed_ctx *ctx);
int lanczos_region_preload(mo_ed_ctx *ctx);
int lanczos_reference_in(mo_ed_ctx *ctx, const Sector &s, const double *h_vec, int nstep,
                         int *nstep_calc, double *a, double *b, void *scratch, size_t cap);
int diag_sector(mo_ed_ctx *ctx, const Sector &s, int nev, std::vector<double> &vals,
                std::vector<DevBuf> *vecs);
// FP64 refinement of an FP32 eigenvector (short FP64 Lanczos + Rayleigh-Ritz
// from it); out gets Dpad doubles, res the final Ritz residual.
int refine_fp64(mo_ed_ctx *ctx, const Sector &s, const float *x, DevBuf &out, double *res);

// ---- Green's function (green.cu) ---------------------------------------------
int apply_c_dev(mo_ed_ctx *ctx, const Sector &in, const Sector &out, int prec, const void *x,
                void *y, int pm, int iorb, int ispin);
int calc_green(mo_ed_ctx *ctx, double *Gr);

// ---- fit (fit.cu) ------------------------------------------------------------
int chi2_grad_dev(mo_ed_ctx *ctx, int nbatch, const double *x, int nwloc, int ns, int nxsize,
                  const double *omega, const double *dev, int nbath, int norb, double *f,
                  double *g, int want_grad);

}  // namespace moed
