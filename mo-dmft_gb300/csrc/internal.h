// internal.h -- shared declarations of the GB300 ED solver (sm_103a).
//
// Data layout in HBM
//   A sector vector X of dimension D = nup*ndown is stored on the device as
//   ndown rows (down-spin ranks in the reference's order, ed_basis.F90:120-123)
//   of row stride ld.  Within a row the up-spin ranks are permuted into
//   "conserved-block order": hybridisation keeps the electron count of every
//   conserved subsystem (an impurity orbital with the bath levels coupled to
//   it), so the up-spin words with equal counts (a block) are closed under
//   up-spin moves.  Blocks are stored one after the other, each padded to a
//   multiple of 4 columns (16-byte aligned starts); inside a block the column
//   index is the mixed-radix number of the subsystems' local states, the last
//   subsystem fastest.  Species::pos maps an up rank to its column,
//   Species::rank_at a column back to its rank (-1 on pads, which are zero).
//   Host entry points convert to and from the reference layout on the device
//   through a staging buffer.
//
//   Per spin species (nsite sites, N electrons) the device holds the words,
//   the inverse rank table, the column permutation and the H*v tables of
//   both roles: as the up spin (columns) the conflict-free gather schedule of
//   every block, the species diagonal and impurity pattern per column and the
//   spin-flip / pair-hop partner columns; as the down spin (rows) the "row
//   sets" -- rows of a block with equal local states in its leading
//   subsystems -- with their moves split into moves inside the set and moves
//   to other rows.
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
constexpr int kMaxSub = 8;        // conserved subsystems handled by the block layout
constexpr int kMaxCoef = 1 + 2 * kMaxHop;   // coupling table: 0, then +-V per coupling

// An up-spin block as the kernel sees it: first column, padded width, first
// schedule header (4 per 128-column chunk, one per column k = 0..3 of a quad).
struct UpBlock {
    int col0, W4, hdr0, W;
    // the block's gather schedule in 16-bit form (0 bytes when a target or a
    // coupling index does not fit): offset in 16-byte units into
    // Species::sched16 and size.  Layout: one word per (64-column chunk, k) =
    // first entry (in entries from the first entry word) << 8 | slots, then
    // the entries: target column | coupling index << 10.
    int s16_off, s16_bytes, pad0, pad1;
};

// Row-set geometry of one down-spin block (host): at level j the rows are
// grouped by the local states of the first j subsystems in the block's row
// axis order; level nsub is one row per set.
struct DownBlock {
    int size;                     // rows in the block
    int rs0[kMaxSub + 1];         // first row set of each level
    int rs_rows[kMaxSub + 1];     // rows per set at each level
    int nset[kMaxSub + 1];        // sets at each level
    int blob_max[kMaxSub + 1];    // largest metadata blob of a set at each level (bytes)
    int cnt[kMaxSub];             // electrons per subsystem (block key)
};

// Metadata blob of one row set (16-byte aligned sections), copied into
// shared memory with the tile:
//   int4 header {rows g, byte offset of the moves, byte offset of the
//                4-operator terms, total bytes}
//   int4 info[g] {impurity pattern | moves in the set << 8 | moves to other
//                 rows << 16 | 4-operator terms << 24, first move, first
//                 4-operator term, row rank}
//   double diag[g]    species diagonal of the row
//   unsigned moves[]  row (index within the set for moves inside it, rank
//                     otherwise) | coupling index << 16; moves inside the set first
//   unsigned q4[]     4-operator terms: partner rank | pair << 16 | pair hop
//                     << 21 | negative sign << 22 (spin-flip uses T_{j<-i},
//                     pair hop T_{i<-j} of the row)

struct Species {
    int nsite = 0, N = 0, n = 0;
    int nsub = 0;
    int ncol = 0;                 // sum of padded block widths
    int ld = 0;                   // row stride when this species is the up spin (roundup(ncol, 32))
    int *words = nullptr;         // [n] ascending words (device)
    int *rank = nullptr;          // [2^nsite] rank of a word, -1 outside the species
    int *pos = nullptr;           // [n] column of each rank
    int *rank_at = nullptr;       // [ld] rank at each column, -1 on pads
    std::vector<int> h_words, h_pos, h_rank_at;
    // ---- up-spin role (columns) ----
    std::vector<UpBlock> h_ublk;
    std::vector<int> h_ublk_cnt;  // [nblk * kMaxSub] electrons per subsystem
    UpBlock *ublk = nullptr;
    // gather schedule: header (block, 64-column chunk, k) = {first entry,
    // slots}; entry (slot s, quad l) at first + 16*s + l = target column
    // within the block | coupling index << 16 (index 0: no move, coupling 0)
    // of column 4*l + k of the chunk.  The 16 targets of one slot are
    // distinct mod 16: with shared-memory row pitches = 16 (mod 32), the two
    // half-warps reading two rows hit 32 different banks.
    int2 *sched_hdr = nullptr;
    unsigned *sched_ent = nullptr;
    int sched_slots_max = 0;
    unsigned char *sched16 = nullptr;   // 16-bit schedules of the blocks (UpBlock::s16_off)
    double *up_diag_d = nullptr;  // [ld] species diagonal per column (pads 0)
    float *up_diag_f = nullptr;
    unsigned char *up_imp = nullptr;  // [ld] impurity pattern per column
    // [npair][ld] up transfer T_{i<-j} of pair p = (i,j) per column: bit 31
    // valid, bit 30 negative sign, low 16 bits the partner column
    unsigned *up4 = nullptr;
    // ---- down-spin role (rows) ----
    std::vector<DownBlock> h_dblk;
    int nrs = 0, nrec = 0;
    int2 *rs = nullptr;           // [nrs] {first row record, rows}
    int *rs_row = nullptr;        // [nrec] row (rank)
    int2 *rs_blob = nullptr;      // [nrs] {byte offset / 16, bytes} of the set's metadata blob
    unsigned char *blob = nullptr;
    std::vector<int2> h_rs, h_rs_blob;   // host copies (tile descriptors)
    ~Species();
};

struct Sector {
    int ne_up, ne_down;
    Species *up, *dn;
    long long D() const { return (long long)up->n * dn->n; }     // dimension
    int ld() const { return up->ld; }                              // device row stride
    long long Dpad() const { return (long long)up->ld * dn->n; }   // device elements
};

// ---------------------------------------------------------------------------
// H*v job (one vector of one sector); the kernel walks a list of jobs
// ---------------------------------------------------------------------------
// A tile: one row set of the down species times one up block.
struct HvTile {
    int rs0, rows, blob16, blob_bytes;   // row set: first row record, rows, metadata blob (16-byte units, bytes)
    int col0, W4, hdr0, s16_off;         // up block (UpBlock fields)
    int s16_bytes, ub, pad0, pad1;
};

template <typename TA>
struct HvJobT {
    const void *x;            // input vector (TX), device layout
    void *y;                  // output vector (TY), device layout
    double *dot_partial;      // optional [grid]: per CTA, sum of x*y over its tiles
    const int *active;        // optional device flag: job skipped when *active == 0
    int ld, ncol, nrow;       // row stride, columns covered by blocks (the rest is pad), rows
    int tile0, ntiles;        // this job's tiles in the batch (tile0 set at launch)
    const HvTile *tiles;
    const UpBlock *ublk;
    const int2 *sched_hdr;
    const unsigned *sched_ent;
    const unsigned char *sched16;
    const TA *up_diag;
    const unsigned char *up_imp;
    const unsigned *up4;
    const int2 *rs;
    const int *rs_row;
    const int2 *rs_blob;
    const unsigned char *blob;
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
    int nsub = 0;                  // number of conserved subsystems (<= kMaxSub)
    std::map<int, std::unique_ptr<moed::Species>> species;  // by N

    // statistics of the last eigensolve (mo_ed_diag_stats)
    int diag_cycles = 0;
    long long diag_matvecs = 0;
    double diag_res_est = 0.0, diag_res_true = 0.0;
    double refine_res = 0.0;   // largest Ritz residual of the last FP64 refinement (green_fp64)

    // sectors / omega
    std::vector<int> nelec, nup;
    std::vector<double> omega;

    // results of ed_solve / green
    std::vector<moed::StateVec> states;
    std::vector<moed::GreenRecord> green;
    // square-lattice band of the DMFT self-consistency (mo_ed_set_band_structure)
    moed::DevBuf d_hk;
    int nq = 0;

    // scratch; stage: the reference-layout copy of a host vector on its way
    // to or from the device layout
    moed::DevBuf scratch_a, scratch_b, scratch_part, stage;
    // H*v tile lists per (sector, stage budget): key -> (tiles, count)
    std::map<long long, std::pair<moed::DevBuf, int>> hv_tiles;
    // device word set by a kernel whose bounded wait ran out (0: none)
    moed::DevBuf d_err;
    // eigensolver workspace reused across sectors (Krylov vectors of sectors
    // up to 64 MB per vector, and the projected-problem arrays)
    std::vector<moed::DevBuf> trl_pool, trl_small, rr_pool;
    // autotuned H*v tile shape per (kind, Nup, Ndn), and the timings (ms) of
    // every shape measured when it was chosen (negative: did not fit)
    std::map<long long, int> hv_choice;
    std::map<long long, std::vector<float>> hv_times;
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
// device layout (ndown rows of stride ld, up ranks at their block columns,
// zero pads); es = element size.  The copy goes through a device staging
// area of D elements: `stage` when given (nothing is allocated), else the
// context's staging buffer.
int upload_padded(mo_ed_ctx *ctx, const Sector &s, const void *host, void *dev, size_t es,
                  void *stage = nullptr);
int download_padded(mo_ed_ctx *ctx, const Sector &s, const void *dev, void *host, size_t es,
                    void *stage = nullptr);
// device-side permutations between the reference layout (D contiguous) and
// the device layout
int to_device_layout(mo_ed_ctx *ctx, const Sector &s, const void *ref, void *dev, size_t es);
int to_reference_layout(mo_ed_ctx *ctx, const Sector &s, const void *dev, void *ref, size_t es);
// FP64 host vector (reference layout) -> FP32 device vector (device layout)
int upload_f64_to_f32(mo_ed_ctx *ctx, const Sector &s, const double *host, float *dev, void *stage = nullptr);
int to_device_layout_f64_f32(mo_ed_ctx *ctx, const Sector &s, const double *ref, float *dev);

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
// Fill a job for sector s (x, y device pointers) under tile-shape variant v
// (its tile list must exist: hv_prepare / hv_prepare_rows).
template <typename TA>
void hv_fill_job(const mo_ed_ctx *ctx, const Sector &s, int kind, int v, const void *x, void *y,
                 HvJobT<TA> &job);
// Launch H*v over a host list of jobs (tile0 is assigned here); jobs are
// passed to the kernel by value, so the call can be captured in a CUDA graph.
int hv_launch_f32(mo_ed_ctx *ctx, int v, const HvJobT<float> *jobs, int njobs);
int hv_launch_f64(mo_ed_ctx *ctx, int kind, int v, const HvJobT<double> *jobs, int njobs);
// Tile-shape variant for sector s (autotuned on the first call per shape;
// that first call allocates and synchronizes, so make it before any stream
// capture), its number of dot-product partials (the grid size), and the tile
// list of the sector.
int hv_prepare(mo_ed_ctx *ctx, const Sector &s, int kind, int *v, int *nparts);
// autotuner record of a shape: per variant (RG, threads, MINB, stage rows) and time in ms
int hv_tuning(mo_ed_ctx *ctx, const Sector &s, int kind, int cap, int *nvar, int *shape, float *ms, int *chosen);
// tile list of variant v for a sector batched with the one v was tuned on
int hv_prepare_rows(mo_ed_ctx *ctx, const Sector &s, int kind, int v);
// Lookup only: the variant and tile list that hv_prepare left for this sector
// and kind, or MO_ED_ERR_STATE if it never ran (never tunes or allocates).
int hv_lookup(mo_ed_ctx *ctx, const Sector &s, int kind, int *v, int *nparts);
// Pin the tile-shape variant of a sector and kind (instead of the autotuner's choice).
int hv_set_variant(mo_ed_ctx *ctx, const Sector &s, int kind, int v);
// Convenience: one vector.
int hv_single(mo_ed_ctx *ctx, const Sector &s, int kind, const void *x, void *y);
// Tile list of a sector for tile-shape variant v of `kind` (built once).
int hv_tile_list(mo_ed_ctx *ctx, const Sector &s, int kind, int v, const HvTile **tiles, int *ntiles);

// ---- Krylov (krylov.cu) -----------------------------------------------------
int lanczos_reference(mo_ed_ctx *ctx, const Sector &s, const double *h_vec, int nstep,
                      int *nstep_calc, double *a, double *b);
// The same recurrence with every device buffer carved from the caller's
// region [scratch, scratch + cap) (256-byte aligned).  Needs hv_lookup to
// succeed for the sector; allocates no device memory.  Bytes needed:
size_t lanczos_region_bytes(const Sector &s, int prec, int nstep, int hv_parts);
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
