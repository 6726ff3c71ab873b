// krylov.cuh -- batched Lanczos state shared by krylov.cu and green.cu.
#pragma once

#include "internal.h"

namespace moed {

constexpr int kLzMaxRuns = 24;
constexpr int kVecChunk = 8192;   // elements per item of the elementwise kernels

// One run of the reference recurrence (ed_lanczos.F90:14-68) on the device.
// u[0..2] hold u_{j-2}, u_{j-1}, u_j (unnormalized, ring), w = H u_j.
struct LzRunDev {
    void *u[3];
    void *w;
    long long D;
    int upd_item0, upd_nitems;    // items of the update kernel (kVecChunk elements)
    int hv_item0, hv_nitems;      // items of the H*v kernel
    double *a, *nrm;              // [nstep+1] device
    int *active;                  // 1 while running
    int *nstep_calc;              // device
    double *upd_part, *hv_part;   // partial sums
};

struct LzBatchDev {
    int nrun, total_items;
    LzRunDev run[kLzMaxRuns];
};

// A batch of reference Lanczos runs sharing every launch.  Host-side owner of
// the device buffers; vectors are FP32 or FP64 per `prec`.
struct LzBatch {
    int prec = MO_ED_FP64;
    int nstep = 0;
    std::vector<Sector> sec;
    std::vector<DevBuf> vecs;     // 4 per run
    DevBuf coef;                  // a, nrm per run
    DevBuf flags;                 // active, nstep_calc per run
    DevBuf upd_part, hv_part;
    std::vector<int> upd_item0, upd_nitems, hv_item0, hv_nitems;
    int upd_total = 0, hv_total = 0;
    int hv_variant = 0, hv_rows = 0;   // H*v tile shape shared by all runs
};

// Allocate a batch for the given target sectors; start vectors are written
// by the caller into start_vector(b, r) (device, prec) before lz_run.
int lz_setup(mo_ed_ctx *ctx, LzBatch &b, const std::vector<Sector> &secs, int prec, int nstep);
void *lz_start_vector(LzBatch &b, int r);
// Run the recurrence for all runs; a, b (squared norms, b[0] = 0) and
// nstep_calc returned per run on the host.
int lz_run(mo_ed_ctx *ctx, LzBatch &b, std::vector<std::vector<double>> &a,
           std::vector<std::vector<double>> &bb, std::vector<int> &nstep_calc);

// FP64 sum of x*y over n elements (x, y of the given precisions), into *d_out.
int dot_dev(mo_ed_ctx *ctx, int prec_x, const void *x, int prec_y, const void *y, long long n,
            double *d_out);
int convert_f64_to_f32(mo_ed_ctx *ctx, const double *in, float *out, long long n);
int convert_f32_to_f64(mo_ed_ctx *ctx, const float *in, double *out, long long n);

}  // namespace moed
