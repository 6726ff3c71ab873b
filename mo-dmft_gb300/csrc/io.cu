// io.cu -- the reference's files for eigenpairs and continued-fraction
// coefficients (ed_io.F90:13-147, ed_green.F90:112-115, dos.f90:16-23).
//
// All files are Fortran unformatted sequential files as gfortran writes them:
// every record is framed by its byte length as a 4-byte little-endian integer
// before and after the payload, and LOGICAL is a 4-byte integer (1 = true).
// Records here stay below 2 GiB (the largest sector vector with 15 sites is
// 331 MB), so no record is split into subrecords.
//
//   eigvec-SS-LLL-NNNN  (ed_io.F90:13-31, 140-145; node NNNN = 0000)
//       record 1: nloc (int32); record 2: nloc doubles in the reference's row
//       order (up-spin rank fastest).
//   eigenvalues.dat     (ed_io.F90:33-56, export_eigval)
//       record 1: nev_calc (int32); record 2: nev_calc entries of {ind (int32),
//       eigenvalue (double), Boltzmann factor (double)}, ind = (sector-1)*nev
//       + level.  import_eigval (ed_io.F90:58-98) reads one record per entry,
//       which does not match the writer; the reader here follows the writer.
//   apbpanbn.dat        (ed_green.F90:112-115, 125-128; read by dos.f90)
//       per record: {nstep_calcp, nstep_calcn} (int32), then {iev, iorb
//       (int32), E, prob (double), even (logical), ap(0:np), bp(0:np),
//       an(0:nn), bn(0:nn)}.  nstep_calc = -1 marks a run whose excitation
//       leaves the Fock space; it has no coefficients.
//
// The reference writes every eigenvector of every sector during ed_solve;
// here the kept states (the ones the Green's function reads back) are
// written on request, since the solver keeps them on the device.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>

#include "krylov.cuh"

namespace moed {
namespace {

struct File {
    FILE *f = nullptr;
    explicit File(FILE *p) : f(p) {}
    ~File()
    {
        if (f) fclose(f);
    }
};

bool put_record(FILE *f, const void *data, size_t bytes)
{
    if (bytes > 0x7fffffffu) return false;
    const int32_t m = (int32_t)bytes;
    return fwrite(&m, 4, 1, f) == 1 && (bytes == 0 || fwrite(data, 1, bytes, f) == bytes) && fwrite(&m, 4, 1, f) == 1;
}

// One record into out: 1 = read, 0 = clean end of file, -1 = a short file or
// inconsistent markers.
int get_record(FILE *f, std::vector<unsigned char> &out)
{
    int32_t m0 = 0, m1 = 0;
    const size_t got = fread(&m0, 1, 4, f);
    if (got == 0 && feof(f)) return 0;
    if (got != 4 || m0 < 0) return -1;
    out.resize((size_t)m0);
    if (m0 > 0 && fread(out.data(), 1, (size_t)m0, f) != (size_t)m0) return -1;
    return fread(&m1, 4, 1, f) == 1 && m1 == m0 ? 1 : -1;
}

struct Packer {
    std::vector<unsigned char> b;
    template <typename T>
    void put(const T &v)
    {
        const unsigned char *p = reinterpret_cast<const unsigned char *>(&v);
        b.insert(b.end(), p, p + sizeof(T));
    }
    void put_n(const double *v, size_t n)
    {
        const unsigned char *p = reinterpret_cast<const unsigned char *>(v);
        b.insert(b.end(), p, p + n * sizeof(double));
    }
};

struct Unpacker {
    const std::vector<unsigned char> &b;
    size_t o = 0;
    bool ok = true;
    template <typename T>
    T get()
    {
        T v{};
        if (o + sizeof(T) > b.size()) {
            ok = false;
            return v;
        }
        memcpy(&v, b.data() + o, sizeof(T));
        o += sizeof(T);
        return v;
    }
};

std::string eigvec_name(const std::string &dir, int isector, int ilevel)
{
    char n[64];
    snprintf(n, sizeof n, "eigvec-%02d-%03d-%04d", isector, ilevel, 0);
    return dir.empty() ? std::string(n) : dir + "/" + n;
}

std::string join(const char *dir, const char *name)
{
    const std::string d = dir ? dir : "";
    return d.empty() ? std::string(name) : d + "/" + name;
}

}  // namespace
}  // namespace moed

using namespace moed;

extern "C" {

int mo_ed_export_eigvec(mo_ed_ctx *ctx, const char *dir)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->states.empty()) return fail(ctx, MO_ED_ERR_STATE, "mo_ed_solve has not been run");
    const std::string d = dir ? dir : "";
    const int nev = ctx->opt.nev;
    // eigenvalues.dat (export_eigval)
    {
        File f(fopen(join(dir, "eigenvalues.dat").c_str(), "wb"));
        if (!f.f) return fail(ctx, MO_ED_ERR_ARG, "cannot create eigenvalues.dat");
        const int32_t nc = (int32_t)ctx->states.size();
        Packer p;
        for (const StateVec &st : ctx->states) {
            p.put<int32_t>(st.sector * nev + st.level + 1);
            p.put<double>(st.val);
            p.put<double>(st.pev);
        }
        if (!put_record(f.f, &nc, 4) || !put_record(f.f, p.b.data(), p.b.size()))
            return fail(ctx, MO_ED_ERR_ARG, "write error in eigenvalues.dat");
    }
    // eigvec-SS-LLL-0000 of every kept state (export_eigvec)
    for (const StateVec &st : ctx->states) {
        Sector s;
        if (int rc = get_sector(ctx, ctx->nup[st.sector], ctx->nelec[st.sector] - ctx->nup[st.sector], &s)) return rc;
        const long long D = s.D();
        std::vector<double> h((size_t)D);
        const void *src = st.vec.p;
        DevBuf wide;
        if (st.prec == MO_ED_FP32) {
            if (int rc = dev_alloc(ctx, wide, sizeof(double) * (size_t)s.Dpad())) return rc;
            if (int rc = convert_f32_to_f64(ctx, (const float *)st.vec.p, (double *)wide.p, s.Dpad())) return rc;
            src = wide.p;
        }
        if (int rc = download_padded(ctx, s, src, h.data(), sizeof(double))) return rc;
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const std::string fn = eigvec_name(d, st.sector + 1, st.level + 1);
        File f(fopen(fn.c_str(), "wb"));
        if (!f.f) return fail(ctx, MO_ED_ERR_ARG, "cannot create " + fn);
        const int32_t nloc = (int32_t)D;
        if (!put_record(f.f, &nloc, 4) || !put_record(f.f, h.data(), sizeof(double) * h.size()))
            return fail(ctx, MO_ED_ERR_CAPACITY, "write error in " + fn);
    }
    return MO_ED_OK;
}

int mo_ed_import_eigvec(mo_ed_ctx *ctx, const char *dir, int *nev_calc)
{
    if (!ctx) return MO_ED_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!ctx->have_model || ctx->nup.empty()) return fail(ctx, MO_ED_ERR_STATE, "model or sectors not set");
    const std::string d = dir ? dir : "";
    const int nev = ctx->opt.nev;
    std::vector<int32_t> ind;
    std::vector<double> val, pev;
    {
        File f(fopen(join(dir, "eigenvalues.dat").c_str(), "rb"));
        if (!f.f) return fail(ctx, MO_ED_ERR_ARG, "cannot open eigenvalues.dat");
        std::vector<unsigned char> r1, r2;
        if (get_record(f.f, r1) != 1 || r1.size() != 4 || get_record(f.f, r2) != 1)
            return fail(ctx, MO_ED_ERR_ARG, "eigenvalues.dat: bad record");
        int32_t nc;
        memcpy(&nc, r1.data(), 4);
        if (nc < 1 || r2.size() != (size_t)nc * 20) return fail(ctx, MO_ED_ERR_ARG, "eigenvalues.dat: bad sizes");
        Unpacker u{r2};
        for (int i = 0; i < nc; ++i) {
            ind.push_back(u.get<int32_t>());
            val.push_back(u.get<double>());
            pev.push_back(u.get<double>());
        }
    }
    double Z = 0.0;
    for (double p : pev) Z += p;
    std::vector<StateVec> states;
    for (size_t i = 0; i < ind.size(); ++i) {
        StateVec st;
        st.sector = (ind[i] - 1) / nev;
        st.level = (ind[i] - 1) % nev;
        if (ind[i] < 1 || st.sector >= (int)ctx->nup.size())
            return fail(ctx, MO_ED_ERR_ARG, "eigenvalues.dat: state outside the sector list");
        st.val = val[i];
        st.pev = pev[i];
        st.prob = pev[i] / Z;
        st.prec = ctx->opt.precision;
        Sector s;
        if (int rc = get_sector(ctx, ctx->nup[st.sector], ctx->nelec[st.sector] - ctx->nup[st.sector], &s)) return rc;
        const std::string fn = eigvec_name(d, st.sector + 1, st.level + 1);
        File f(fopen(fn.c_str(), "rb"));
        if (!f.f) return fail(ctx, MO_ED_ERR_ARG, "import_eigvec: file not found, " + fn);
        std::vector<unsigned char> r1, r2;
        if (get_record(f.f, r1) != 1 || r1.size() != 4 || get_record(f.f, r2) != 1)
            return fail(ctx, MO_ED_ERR_ARG, fn + ": bad record");
        int32_t nloc;
        memcpy(&nloc, r1.data(), 4);
        if ((long long)nloc != s.D() || r2.size() != (size_t)nloc * sizeof(double))
            return fail(ctx, MO_ED_ERR_ARG, fn + ": basis dimension mismatch");
        DevBuf wide;
        if (int rc = dev_alloc(ctx, wide, sizeof(double) * (size_t)s.Dpad())) return rc;
        if (int rc = upload_padded(ctx, s, r2.data(), wide.p, sizeof(double))) return rc;
        if (st.prec == MO_ED_FP32) {
            if (int rc = dev_alloc(ctx, st.vec, sizeof(float) * (size_t)s.Dpad())) return rc;
            if (int rc = convert_f64_to_f32(ctx, (const double *)wide.p, (float *)st.vec.p, s.Dpad())) return rc;
        } else {
            st.vec = std::move(wide);
        }
        MOED_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        states.push_back(std::move(st));
    }
    ctx->states = std::move(states);
    ctx->green.clear();
    if (nev_calc) *nev_calc = (int)ctx->states.size();
    return MO_ED_OK;
}

int mo_ed_write_apbpanbn(mo_ed_ctx *ctx, const char *path)
{
    if (!ctx || !path) return MO_ED_ERR_ARG;
    if (ctx->green.empty()) return fail(ctx, MO_ED_ERR_STATE, "mo_ed_calc_green_ftn has not been run");
    File f(fopen(path, "wb"));
    if (!f.f) return fail(ctx, MO_ED_ERR_ARG, std::string("cannot create ") + path);
    for (const GreenRecord &g : ctx->green) {
        const int32_t ns[2] = {g.np, g.nn};
        Packer p;
        p.put<int32_t>(g.iev);
        p.put<int32_t>(g.iorb);
        p.put<double>(g.val);
        p.put<double>(g.prob);
        p.put<int32_t>(g.even ? 1 : 0);
        p.put_n(g.ap.data(), (size_t)(g.np + 1));
        p.put_n(g.bp.data(), (size_t)(g.np + 1));
        p.put_n(g.an.data(), (size_t)(g.nn + 1));
        p.put_n(g.bn.data(), (size_t)(g.nn + 1));
        if (!put_record(f.f, ns, sizeof ns) || !put_record(f.f, p.b.data(), p.b.size()))
            return fail(ctx, MO_ED_ERR_ARG, std::string("write error in ") + path);
    }
    return MO_ED_OK;
}

int mo_ed_read_apbpanbn(mo_ed_ctx *ctx, const char *path, int *nrec)
{
    if (!ctx || !path) return MO_ED_ERR_ARG;
    if (!ctx->have_model) return fail(ctx, MO_ED_ERR_STATE, "model not set");
    File f(fopen(path, "rb"));
    if (!f.f) return fail(ctx, MO_ED_ERR_ARG, std::string("cannot open ") + path);
    const int ld = ctx->opt.nstep + 1;
    std::vector<GreenRecord> recs;
    std::vector<unsigned char> r1, r2;
    for (;;) {
        const int rc1 = get_record(f.f, r1);
        if (rc1 == 0) break;
        if (rc1 < 0 || r1.size() != 8 || get_record(f.f, r2) != 1)
            return fail(ctx, MO_ED_ERR_ARG, "apbpanbn: bad or truncated record");
        int32_t ns[2];
        memcpy(ns, r1.data(), 8);
        if (ns[0] < -1 || ns[1] < -1 || ns[0] >= ld || ns[1] >= ld)
            return fail(ctx, MO_ED_ERR_ARG, "apbpanbn: nstep_calc beyond the context's nstep");
        Unpacker u{r2};
        GreenRecord g;
        g.np = ns[0];
        g.nn = ns[1];
        g.iev = u.get<int32_t>();
        g.iorb = u.get<int32_t>();
        g.val = u.get<double>();
        g.prob = u.get<double>();
        g.even = u.get<int32_t>() != 0;
        if (g.iorb < 1 || g.iorb > ctx->norb) return fail(ctx, MO_ED_ERR_ARG, "apbpanbn: orbital out of range");
        std::vector<double> *dst[4] = {&g.ap, &g.bp, &g.an, &g.bn};
        for (int k = 0; k < 4; ++k) {
            dst[k]->assign(ld, 0.0);
            const int n = (k < 2 ? g.np : g.nn) + 1;
            for (int j = 0; j < n; ++j) (*dst[k])[j] = u.get<double>();
        }
        if (!u.ok || u.o != r2.size()) return fail(ctx, MO_ED_ERR_ARG, "apbpanbn: record length mismatch");
        recs.push_back(std::move(g));
    }
    ctx->green = std::move(recs);
    if (nrec) *nrec = (int)ctx->green.size();
    return MO_ED_OK;
}

}  // extern "C"
