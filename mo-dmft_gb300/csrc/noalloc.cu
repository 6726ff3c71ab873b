// noalloc.cu -- the Lanczos recurrence for hosts that cannot allocate device
// memory while they run.
//
// A DMFT driver that hands the whole GPU to its own memory pool up front (the
// arrays of its self-consistency loop: Green's functions, hybridisations,
// bath parameters), or whose outer loop cannot stand the device-wide
// synchronisation that cudaFree implies, still needs the Lanczos
// coefficients of each excitation.  mo_ed_lanczos_iteration allocates its
// Krylov vectors, coefficients and partial sums on every call;
// mo_ed_lanczos_iteration_noalloc runs the same kernels on a fixed region
// that the library reserves statically on every GPU that loads it.
//
// The region is kNoAllocBytes (32 MiB) and is held until the process exits.
// It fits sectors up to about 1.0e6 padded elements in FP64 and 2.0e6 in
// FP32 (4 vectors, with the FP64 start vector staged in two of the FP32
// ones); larger sectors get MO_ED_ERR_CAPACITY.  Every call shares it and it
// keeps the previous call's contents: the coefficients and flags are
// cleared by each call before use, and every vector element is written
// before it is read.  Calls that overlap on the GPU (two contexts, streams or
// host threads at once) race on the region and must be serialised by the
// caller.
#include "internal.h"

#include <mutex>

namespace {
constexpr size_t kNoAllocBytes = (size_t)32 << 20;
constexpr int kNoAllocMaxDevices = 64;
}  // namespace

// Device region of the no-allocation entry point.  In host code this name is
// only a handle for cudaGetSymbolAddress, not a device address.
static __device__ __align__(256) unsigned char mo_ed_noalloc_region[kNoAllocBytes];

namespace {
std::mutex g_region_mu;
void *g_region_addr[kNoAllocMaxDevices];

// Device address of the region on the context's device; looked up once per
// device, with that device current.  mo_ed_create does the look-up, so the
// region is committed on the device when the first context on it is created
// (lazy module loading would otherwise load the module, and reserve the 32
// MiB, on the first no-allocation call).  The cached address belongs to the
// device's primary context: a device reset after the look-up is not
// supported.
int region_address(mo_ed_ctx *ctx, void **out)
{
    if (ctx->device < 0 || ctx->device >= kNoAllocMaxDevices)
        return moed::fail(ctx, MO_ED_ERR_ARG, "device ordinal beyond the no-allocation table");
    std::lock_guard<std::mutex> lock(g_region_mu);
    if (!g_region_addr[ctx->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, mo_ed_noalloc_region);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return moed::cuda_fail(ctx, e, "cudaGetSymbolAddress");
        }
        g_region_addr[ctx->device] = p;
    }
    *out = g_region_addr[ctx->device];
    return MO_ED_OK;
}
}  // namespace

namespace moed {
int noalloc_prepare(mo_ed_ctx *ctx)
{
    void *p = nullptr;
    if (int rc = region_address(ctx, &p)) return rc;
    return lanczos_region_preload(ctx);
}
}  // namespace moed

using namespace moed;

extern "C" {

int mo_ed_lanczos_iteration_noalloc(mo_ed_ctx *ctx, int ne_up, int ne_down, const double *vec,
                                    int *nstep_calc, double *a, double *b)
{
    if (!ctx) return MO_ED_ERR_ARG;
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        cudaGetLastError();
        return fail(ctx, MO_ED_ERR_CUDA, "cannot make the context's device current");
    }
    if (!vec || !nstep_calc || !a || !b) return fail(ctx, MO_ED_ERR_ARG, "bad arguments");
    Sector s;
    if (int rc = find_sector(ctx, ne_up, ne_down, &s)) return rc;
    const int prec = ctx->opt.precision;
    int v = 0, R = 0;
    if (int rc = hv_lookup(ctx, s, prec == MO_ED_FP32 ? HV_F32 : HV_F64, &v, &R)) return rc;
    const int nstep = ctx->opt.nstep;
    const size_t need = lanczos_region_bytes(s, prec, nstep, R);
    if (need > kNoAllocBytes)
        return fail(ctx, MO_ED_ERR_CAPACITY,
                    "sector needs " + std::to_string(need) + " bytes, the no-allocation region holds " +
                        std::to_string(kNoAllocBytes));
    void *region = nullptr;
    if (int rc = region_address(ctx, &region)) return rc;
    return lanczos_reference_in(ctx, s, vec, nstep, nstep_calc, a, b, region, kNoAllocBytes);
}

}  // extern "C"
