// netCDF output of cell and surface properties: NCDataHolder / write_netcdf /
// close_netcdf for PhysProps (io.jl:116-330) and NCDataHolderSurf /
// write_netcdf for SurfProps (io.jl:430-600).
//
// Container: netCDF classic, 64-bit offset variant ("CDF-2", Unidata's
// published classic format specification), big-endian.  The dimensions,
// variables (names, types, dimension order), skip lists and the ndens comment
// attribute are the reference's; it writes the netCDF-4 (HDF5) container,
// which needs the HDF5 library.  Classic netCDF has no string type, so
// species_names is a char variable (n_species, species_name_length), and no
// fixed dimension of length 0, so a property set without moments has neither
// the n_moments dimension nor the moment variables.
//
// One time step of a classic file is one contiguous record (every record
// variable's slab in definition order), so an output step is a single append:
//   1. k_nc_pack (on the context's stream, after the kernels that computed the
//      properties) packs the record big-endian into the slot's device buffer;
//   2. a side stream copies it into the slot's pinned host buffer;
//   3. the file's writer thread waits for the copy, writes the record at its
//      offset and then the record count in the header (readers never see a
//      partial record), and syncs every sync_freq records.
// The caller's time loop does not wait for the disk; it waits only when all
// slots are still being written.
#include "cell_ops.cuh"
#include "mz_host.h"

#include <fcntl.h>
#include <unistd.h>

#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>

namespace {

enum : uint32_t { T_CHAR = 2, T_INT = 4, T_DOUBLE = 6 };
enum : uint32_t { TAG_DIM = 0x0A, TAG_VAR = 0x0B, TAG_ATT = 0x0C };
constexpr int NC_SLOTS = 3;
constexpr int MAX_SEGS = 10;

// one piece of a record: n doubles from device memory (contiguous, or gathered
// from a surface set's per-(species, wall) sums), or from inline host values
struct PackSeg {
    const double* src;  // null: take inl[inl_off ...]
    int64_t n;
    int64_t dst;      // offset in doubles within the record
    int32_t qbase;    // surface gather: first quantity index, -1 = contiguous
    int32_t ncomp;    // surface gather: components per (wall, species)
    int32_t inl_off;
};

struct PackArgs {
    PackSeg seg[MAX_SEGS];
    int32_t nseg;
    double inl[1 + MZ_MAX_SPECIES];
};

__device__ __forceinline__ uint64_t be64(double x)
{
    const uint32_t lo = (uint32_t)__double2loint(x), hi = (uint32_t)__double2hiint(x);
    return ((uint64_t)__byte_perm(lo, 0, 0x0123) << 32) | (uint64_t)__byte_perm(hi, 0, 0x0123);
}

__global__ void k_nc_pack(PackArgs a, uint64_t* out)
{
    for (int k = 0; k < a.nseg; ++k) {
        const PackSeg s = a.seg[k];
        for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < s.n; i += (int64_t)gridDim.x * blockDim.x) {
            double v;
            if (!s.src) {
                v = a.inl[s.inl_off + i];
            } else if (s.qbase < 0) {
                v = s.src[i];
            } else {
                const int64_t comp = i % s.ncomp, ix = i / s.ncomp;  // ix = wall + 2 species
                v = s.src[ix * mz::SURF_Q + s.qbase + comp];
            }
            out[s.dst + i] = be64(v);
        }
    }
}

uint64_t host_be64(double x)
{
    uint64_t u;
    memcpy(&u, &x, 8);
    uint64_t r = 0;
    for (int b = 0; b < 8; ++b) r |= ((u >> (8 * b)) & 0xFFu) << (8 * (7 - b));
    return r;
}

// big-endian header serialiser
struct Bytes {
    std::vector<uint8_t> b;
    void u32(uint32_t v)
    {
        for (int k = 3; k >= 0; --k) b.push_back((uint8_t)(v >> (8 * k)));
    }
    void u64(uint64_t v)
    {
        for (int k = 7; k >= 0; --k) b.push_back((uint8_t)(v >> (8 * k)));
    }
    void pad()
    {
        while (b.size() % 4) b.push_back(0);
    }
    void name(const std::string& s)
    {
        u32((uint32_t)s.size());
        b.insert(b.end(), s.begin(), s.end());
        pad();
    }
};

struct Attr {
    std::string name;
    uint32_t type;
    uint32_t count;
    std::vector<uint8_t> data;  // big-endian values
};

struct Var {
    std::string name;
    std::vector<int> dims;  // dimension ids, slowest first
    uint32_t type;
    bool rec;
    uint64_t vsize = 0, begin = 0;
};

// which property a record variable holds
enum Field { F_TIMESTEP, F_LPA, F_MOMENTS, F_NP, F_NDENS, F_V, F_T, F_SNP, F_FLUX_IN, F_FLUX_OUT, F_FORCE, F_PN,
             F_SHEAR, F_KEF };

bool in_list(const char* const* list, int32_t n, const char* a, const char* b = nullptr)
{
    for (int32_t i = 0; i < n; ++i)
        if (list[i] && (!strcmp(list[i], a) || (b && !strcmp(list[i], b)))) return true;
    return false;
}

}  // namespace

struct mz_nc_file_s {
    mz_ctx* ctx = nullptr;
    bool surf = false;
    int32_t n_cells = 0, n_species = 0, n_moments = 0, n_elements = 0, ndens_not_Np = 0;
    std::string path, last_error;
    int fd = -1;
    uint64_t rec_begin = 0, recsize = 0;  // bytes
    uint32_t numrecs = 0;                 // records queued
    std::vector<std::pair<Field, int64_t>> fields;  // record layout: field, doubles

    struct Slot {
        uint64_t* host = nullptr;  // pinned when ctx, else plain
        uint64_t* dev = nullptr;
        cudaEvent_t ready = nullptr;
        bool from_device = false;
        bool busy = false;
        uint32_t rec = 0;
        int32_t sync_freq = 0;
    };
    Slot slot[NC_SLOTS];
    int next_slot = 0;
    cudaStream_t copy_stream = nullptr;

    std::thread th;
    std::mutex m;
    std::condition_variable cv;
    std::deque<int> queue;
    bool stop = false;
    std::string io_error;  // set by the writer thread
};

namespace {

void write_all(int fd, const void* p, size_t n, uint64_t off)
{
    const uint8_t* c = (const uint8_t*)p;
    while (n) {
        const ssize_t w = pwrite(fd, c, n, (off_t)off);
        if (w <= 0) throw MzError(MZ_E_ARG, std::string("netCDF write failed: ") + strerror(errno));
        c += w;
        n -= (size_t)w;
        off += (uint64_t)w;
    }
}

void writer_loop(mz_nc_file_s* f)
{
    if (f->ctx) cudaSetDevice(f->ctx->device);
    for (;;) {
        int k;
        {
            std::unique_lock<std::mutex> lk(f->m);
            f->cv.wait(lk, [&] { return f->stop || !f->queue.empty(); });
            if (f->queue.empty()) return;
            k = f->queue.front();
        }
        auto& s = f->slot[k];
        std::string err;
        try {
            if (s.from_device) {
                const cudaError_t e = cudaEventSynchronize(s.ready);
                if (e != cudaSuccess) throw MzError(MZ_E_CUDA, cudaGetErrorString(e));
            }
            write_all(f->fd, s.host, f->recsize, f->rec_begin + (uint64_t)s.rec * f->recsize);
            Bytes n;
            n.u32(s.rec + 1);
            write_all(f->fd, n.b.data(), 4, 4);
            if (s.sync_freq > 0 && (s.rec + 1) % (uint32_t)s.sync_freq == 0) fsync(f->fd);
        } catch (std::exception& e) {
            err = e.what();
        }
        {
            std::lock_guard<std::mutex> lk(f->m);
            if (!err.empty() && f->io_error.empty()) f->io_error = err;
            f->queue.pop_front();
            s.busy = false;
        }
        f->cv.notify_all();
    }
}

// header, fixed variables and writer thread of a new file
void nc_open(mz_nc_file_s* f, const std::vector<std::pair<std::string, uint32_t>>& dims,
             std::vector<Attr>& gatts, std::vector<Var>& vars, const std::vector<std::vector<uint8_t>>& fixed_data)
{
    // sizes
    uint64_t recsize = 0;
    for (auto& v : vars) {
        uint64_t n = v.type == T_DOUBLE ? 8 : v.type == T_INT ? 4 : 1;
        for (int d : v.dims)
            if (dims[d].second) n *= dims[d].second;
        v.vsize = (n + 3) / 4 * 4;
        if (v.rec) recsize += v.vsize;
    }
    auto header = [&]() {
        Bytes h;
        h.b = {'C', 'D', 'F', 2};
        h.u32(0);  // numrecs
        h.u32(TAG_DIM);
        h.u32((uint32_t)dims.size());
        for (auto& d : dims) {
            h.name(d.first);
            h.u32(d.second);
        }
        if (gatts.empty()) {
            h.u32(0);
            h.u32(0);
        } else {
            h.u32(TAG_ATT);
            h.u32((uint32_t)gatts.size());
            for (auto& a : gatts) {
                h.name(a.name);
                h.u32(a.type);
                h.u32(a.count);
                h.b.insert(h.b.end(), a.data.begin(), a.data.end());
                h.pad();
            }
        }
        h.u32(TAG_VAR);
        h.u32((uint32_t)vars.size());
        for (auto& v : vars) {
            h.name(v.name);
            h.u32((uint32_t)v.dims.size());
            for (int d : v.dims) h.u32((uint32_t)d);
            h.u32(0);  // no variable attributes
            h.u32(0);
            h.u32(v.type);
            h.u32(v.vsize > 0xFFFFFFFCull ? 0xFFFFFFFFu : (uint32_t)v.vsize);
            h.u64(v.begin);
        }
        return h;
    };
    const uint64_t hsize = header().b.size();
    uint64_t off = hsize;
    for (auto& v : vars)
        if (!v.rec) {
            v.begin = off;
            off += v.vsize;
        }
    f->rec_begin = off;
    for (auto& v : vars)
        if (v.rec) {
            v.begin = off;
            off += v.vsize;
        }
    f->recsize = recsize;
    f->fd = open(f->path.c_str(), O_WRONLY | O_CREAT | O_TRUNC, 0644);
    if (f->fd < 0) throw MzError(MZ_E_ARG, "cannot create " + f->path + ": " + strerror(errno));
    const Bytes h = header();
    write_all(f->fd, h.b.data(), h.b.size(), 0);
    size_t fi = 0;
    for (auto& v : vars)
        if (!v.rec) {
            std::vector<uint8_t> d = fixed_data.at(fi++);
            d.resize(v.vsize, 0);
            write_all(f->fd, d.data(), d.size(), v.begin);
        }
    for (int k = 0; k < NC_SLOTS; ++k) {
        auto& s = f->slot[k];
        if (f->ctx) {
            MZ_CK(cudaMallocHost(&s.host, recsize));
            MZ_CK(cudaMalloc(&s.dev, recsize));
            MZ_CK(cudaEventCreateWithFlags(&s.ready, cudaEventDisableTiming));
        } else {
            s.host = (uint64_t*)malloc(recsize);
            if (!s.host) throw MzError(MZ_E_NOMEM, "netCDF record buffer");
        }
    }
    if (f->ctx) MZ_CK(cudaStreamCreateWithFlags(&f->copy_stream, cudaStreamNonBlocking));
    f->th = std::thread(writer_loop, f);
}

Attr text_attr(const std::string& name, const std::string& text)
{
    Attr a{name, T_CHAR, (uint32_t)text.size(), std::vector<uint8_t>(text.begin(), text.end())};
    return a;
}

void user_attrs(std::vector<Attr>& out, const mz_nc_attribute* g, int32_t n)
{
    for (int32_t i = 0; i < n; ++i) {
        MZ_REQUIRE(g[i].name && g[i].values && g[i].count >= 0, "netCDF attribute: bad entry");
        Attr a{g[i].name, 0, (uint32_t)g[i].count, {}};
        Bytes b;
        if (g[i].type == MZ_NC_ATTR_TEXT) {
            a.type = T_CHAR;
            const char* t = (const char*)g[i].values;
            b.b.assign(t, t + g[i].count);
        } else if (g[i].type == MZ_NC_ATTR_INT) {
            a.type = T_INT;
            for (int32_t k = 0; k < g[i].count; ++k) b.u32((uint32_t)((const int32_t*)g[i].values)[k]);
        } else if (g[i].type == MZ_NC_ATTR_DOUBLE) {
            a.type = T_DOUBLE;
            for (int32_t k = 0; k < g[i].count; ++k) {
                uint64_t bits;
                memcpy(&bits, (const double*)g[i].values + k, 8);
                b.u64(bits);
            }
        } else {
            throw MzError(MZ_E_ARG, "netCDF attribute: unknown type");
        }
        a.data = b.b;
        out.push_back(a);
    }
}

// species_names as (n_species, species_name_length) chars, zero padded; the
// reference writes the names of species_data into the n_species entries of
// the property set, so fewer names than entries leave the rest empty
std::vector<uint8_t> names_block(const char* const* names, int32_t n_names, int32_t ns, uint32_t& len)
{
    MZ_REQUIRE(n_names >= 0 && n_names <= ns && (n_names == 0 || names), "netCDF: more species names than species");
    len = 1;
    for (int32_t s = 0; s < n_names; ++s) {
        MZ_REQUIRE(names[s], "netCDF: species name missing");
        len = std::max<uint32_t>(len, (uint32_t)strlen(names[s]));
    }
    std::vector<uint8_t> d((size_t)ns * len, 0);
    for (int32_t s = 0; s < n_names; ++s) memcpy(d.data() + (size_t)s * len, names[s], strlen(names[s]));
    return d;
}

// take a free slot (waits while the writer thread still holds all of them)
int acquire_slot(mz_nc_file_s* f)
{
    std::unique_lock<std::mutex> lk(f->m);
    const int k = f->next_slot;
    f->cv.wait(lk, [&] { return !f->slot[k].busy; });
    if (!f->io_error.empty()) throw MzError(MZ_E_ARG, f->io_error);
    f->next_slot = (k + 1) % NC_SLOTS;
    return k;
}

void submit_slot(mz_nc_file_s* f, int k, bool from_device, int32_t sync_freq)
{
    {
        std::lock_guard<std::mutex> lk(f->m);
        auto& s = f->slot[k];
        s.busy = true;
        s.from_device = from_device;
        s.rec = f->numrecs++;
        s.sync_freq = sync_freq;
        f->queue.push_back(k);
    }
    f->cv.notify_all();
}

// enqueue the device record: pack on the context stream, copy on the side stream
void device_record(mz_nc_file_s* f, int k, PackArgs& a)
{
    mz_ctx* c = f->ctx;
    MZ_CK(cudaSetDevice(c->device));
    auto& s = f->slot[k];
    const int64_t nd = (int64_t)(f->recsize / 8);
    const int blocks = (int)std::min<int64_t>(std::max<int64_t>(div_up(nd, 256), 1), 4 * (int64_t)c->num_sms);
    MZ_LAUNCH(c, "nc_pack", k_nc_pack, blocks, 256, 0, a, s.dev);
    MZ_CK(cudaEventRecord(s.ready, c->stream));
    MZ_CK(cudaStreamWaitEvent(f->copy_stream, s.ready, 0));
    MZ_CK(cudaMemcpyAsync(s.host, s.dev, f->recsize, cudaMemcpyDeviceToHost, f->copy_stream));
    MZ_CK(cudaEventRecord(s.ready, f->copy_stream));
}

void host_record(mz_nc_file_s* f, int k, const std::vector<const double*>& src)
{
    uint64_t* out = f->slot[k].host;
    int64_t o = 0;
    for (size_t i = 0; i < f->fields.size(); ++i) {
        const int64_t n = f->fields[i].second;
        MZ_REQUIRE(src[i], "netCDF write: a written variable's array is NULL");
        for (int64_t j = 0; j < n; ++j) out[o + j] = host_be64(src[i][j]);
        o += n;
    }
}

void drain(mz_nc_file_s* f)
{
    std::unique_lock<std::mutex> lk(f->m);
    f->cv.wait(lk, [&] { return f->queue.empty(); });
}

void report(mz_nc_file_s* f, const std::string& m)
{
    f->last_error = m;
    if (f->ctx) set_err(f->ctx, m);
}

}  // namespace

extern "C" {

int mz_nc_props_create(const char* path, const char* const* skip, int32_t n_skip, const char* const* species_names,
                       int32_t n_names, int32_t n_species, int32_t n_cells, int32_t n_moments, const int32_t* moment_powers,
                       int32_t ndens_not_Np, const mz_nc_attribute* gatts, int32_t n_gatts, mz_ctx* ctx,
                       mz_nc_file** out)
{
    if (!out) return MZ_E_ARG;
    *out = nullptr;
    mz_nc_file_s* f = nullptr;
    try {
        MZ_REQUIRE(path && n_species > 0 && n_species <= MZ_MAX_SPECIES && n_cells > 0 && n_moments >= 0 &&
                       (n_moments == 0 || moment_powers) && n_skip >= 0 && (n_skip == 0 || skip),
                   "mz_nc_props_create: bad argument");
        f = new mz_nc_file_s();
        f->ctx = ctx;
        f->path = path;
        f->n_cells = n_cells;
        f->n_species = n_species;
        f->n_moments = n_moments;
        f->ndens_not_Np = ndens_not_Np ? 1 : 0;
        // IOSkipList (io.jl:19-80)
        const bool sk_lpa = in_list(skip, n_skip, "length_particle_array");
        const bool sk_mom = in_list(skip, n_skip, "moments") || n_moments == 0;
        const bool sk_np = in_list(skip, n_skip, "np", "nparticles");
        const bool sk_nd = in_list(skip, n_skip, "ndens");
        const bool sk_v = in_list(skip, n_skip, "v");
        const bool sk_T = in_list(skip, n_skip, "T");

        std::vector<Attr> ga;
        user_attrs(ga, gatts, n_gatts);
        ga.push_back(text_attr("COMMENT ndens",
                               f->ndens_not_Np
                                   ? "In this file, the ndens variable stores the number density, NOT # of physical "
                                     "particles in cell"
                                   : "In this file, the ndens variable stores # of physical particles in cell, NOT "
                                     "number density"));
        uint32_t slen = 0;
        std::vector<std::vector<uint8_t>> fixed{names_block(species_names, n_names, n_species, slen)};
        // dimensions (io.jl:167-171) + the species-name length
        std::vector<std::pair<std::string, uint32_t>> dims{{"vel_components", 3}, {"n_cells", (uint32_t)n_cells},
                                                           {"n_species", (uint32_t)n_species}};
        const int D_V = 0, D_C = 1, D_S = 2;
        int D_M = -1;
        if (!sk_mom) {
            D_M = (int)dims.size();
            dims.push_back({"n_moments", (uint32_t)n_moments});
        }
        const int D_T = (int)dims.size();
        dims.push_back({"timestep", 0});
        const int D_L = (int)dims.size();
        dims.push_back({"species_name_length", slen});
        // variables in the reference's order (io.jl:173-211); dimension lists
        // slowest first (the reverse of the Julia declaration)
        std::vector<Var> vars;
        vars.push_back({"species_names", {D_S, D_L}, T_CHAR, false});
        vars.push_back({"timestep", {D_T}, T_DOUBLE, true});
        f->fields.push_back({F_TIMESTEP, 1});
        const int64_t cs = (int64_t)n_cells * n_species;
        if (!sk_lpa) {
            vars.push_back({"length_particle_array", {D_T, D_S}, T_DOUBLE, true});
            f->fields.push_back({F_LPA, n_species});
        }
        if (!sk_mom) {
            vars.push_back({"moment_powers", {D_M}, T_INT, false});
            Bytes b;
            for (int32_t k = 0; k < n_moments; ++k) b.u32((uint32_t)moment_powers[k]);
            fixed.push_back(b.b);
            vars.push_back({"moments", {D_T, D_S, D_C, D_M}, T_DOUBLE, true});
            f->fields.push_back({F_MOMENTS, cs * n_moments});
        }
        if (!sk_np) {
            vars.push_back({"np", {D_T, D_S, D_C}, T_DOUBLE, true});
            f->fields.push_back({F_NP, cs});
        }
        if (!sk_nd) {
            vars.push_back({"ndens", {D_T, D_S, D_C}, T_DOUBLE, true});
            f->fields.push_back({F_NDENS, cs});
        }
        if (!sk_v) {
            vars.push_back({"v", {D_T, D_S, D_C, D_V}, T_DOUBLE, true});
            f->fields.push_back({F_V, 3 * cs});
        }
        if (!sk_T) {
            vars.push_back({"T", {D_T, D_S, D_C}, T_DOUBLE, true});
            f->fields.push_back({F_T, cs});
        }
        nc_open(f, dims, ga, vars, fixed);
        *out = f;
        return MZ_OK;
    } catch (MzError& e) {
        if (ctx) set_err(ctx, e.what());
        if (f) mz_nc_close(f);
        return e.code;
    } catch (std::exception& e) {
        if (ctx) set_err(ctx, e.what());
        if (f) mz_nc_close(f);
        return MZ_E_ARG;
    }
}

int mz_nc_surf_create(const char* path, const char* const* skip, int32_t n_skip, const char* const* species_names,
                      int32_t n_names, int32_t n_species, int32_t n_elements, const mz_nc_attribute* gatts, int32_t n_gatts,
                      mz_ctx* ctx, mz_nc_file** out)
{
    if (!out) return MZ_E_ARG;
    *out = nullptr;
    mz_nc_file_s* f = nullptr;
    try {
        MZ_REQUIRE(path && n_species > 0 && n_species <= MZ_MAX_SPECIES && n_elements > 0 && n_skip >= 0 &&
                       (n_skip == 0 || skip),
                   "mz_nc_surf_create: bad argument");
        f = new mz_nc_file_s();
        f->ctx = ctx;
        f->surf = true;
        f->path = path;
        f->n_species = n_species;
        f->n_elements = n_elements;
        // IOSkipListSurf (io.jl:334-418)
        const bool sk_np = in_list(skip, n_skip, "np", "nparticles");
        const bool sk_fl = in_list(skip, n_skip, "fluxes");
        const bool sk_f = in_list(skip, n_skip, "force");
        const bool sk_pn = in_list(skip, n_skip, "normal_pressure");
        const bool sk_sh = in_list(skip, n_skip, "shear_pressure");
        const bool sk_ke = in_list(skip, n_skip, "kinetic_energy_flux");
        std::vector<Attr> ga;
        user_attrs(ga, gatts, n_gatts);
        uint32_t slen = 0;
        std::vector<std::vector<uint8_t>> fixed{names_block(species_names, n_names, n_species, slen)};
        // io.jl:475-478
        std::vector<std::pair<std::string, uint32_t>> dims{{"vector_components", 3},
                                                           {"n_elements", (uint32_t)n_elements},
                                                           {"n_species", (uint32_t)n_species},
                                                           {"timestep", 0},
                                                           {"species_name_length", slen}};
        const int D_V = 0, D_E = 1, D_S = 2, D_T = 3, D_L = 4;
        const int64_t es = (int64_t)n_elements * n_species;
        std::vector<Var> vars;  // io.jl:480-513
        vars.push_back({"species_names", {D_S, D_L}, T_CHAR, false});
        vars.push_back({"timestep", {D_T}, T_DOUBLE, true});
        f->fields.push_back({F_TIMESTEP, 1});
        if (!sk_np) {
            vars.push_back({"np", {D_T, D_S, D_E}, T_DOUBLE, true});
            f->fields.push_back({F_SNP, es});
        }
        if (!sk_fl) {
            vars.push_back({"flux_incident", {D_T, D_S, D_E}, T_DOUBLE, true});
            f->fields.push_back({F_FLUX_IN, es});
            vars.push_back({"flux_reflected", {D_T, D_S, D_E}, T_DOUBLE, true});
            f->fields.push_back({F_FLUX_OUT, es});
        }
        if (!sk_f) {
            vars.push_back({"force", {D_T, D_S, D_E, D_V}, T_DOUBLE, true});
            f->fields.push_back({F_FORCE, 3 * es});
        }
        if (!sk_pn) {
            vars.push_back({"normal_pressure", {D_T, D_S, D_E}, T_DOUBLE, true});
            f->fields.push_back({F_PN, es});
        }
        if (!sk_sh) {
            vars.push_back({"shear_pressure", {D_T, D_S, D_E, D_V}, T_DOUBLE, true});
            f->fields.push_back({F_SHEAR, 3 * es});
        }
        if (!sk_ke) {
            vars.push_back({"kinetic_energy_flux", {D_T, D_S, D_E}, T_DOUBLE, true});
            f->fields.push_back({F_KEF, es});
        }
        nc_open(f, dims, ga, vars, fixed);
        *out = f;
        return MZ_OK;
    } catch (MzError& e) {
        if (ctx) set_err(ctx, e.what());
        if (f) mz_nc_close(f);
        return e.code;
    } catch (std::exception& e) {
        if (ctx) set_err(ctx, e.what());
        if (f) mz_nc_close(f);
        return MZ_E_ARG;
    }
}

int mz_nc_props_write(mz_nc_file* f, const mz_props* p, double timestep, int32_t sync_freq)
{
    if (!f) return MZ_E_ARG;
    try {
        MZ_REQUIRE(!f->surf && p && f->ctx && p->dom->ctx == f->ctx, "mz_nc_props_write: bad argument");
        const mz_domain* d = p->dom;
        MZ_REQUIRE(d->n_cells == f->n_cells && d->ns == f->n_species, "mz_nc_props_write: shape differs from the file");
        MZ_REQUIRE((p->ndens != 0) == (f->ndens_not_Np != 0),
                   "Inconsistent computation of ndens/number of physical particles in cell");
        PackArgs a;
        memset(&a, 0, sizeof a);
        a.inl[0] = timestep;
        for (int s = 0; s < f->n_species; ++s) a.inl[1 + s] = p->lpa[s];
        int64_t off = 0;
        for (auto& fl : f->fields) {
            PackSeg& s = a.seg[a.nseg++];
            s.n = fl.second;
            s.dst = off;
            s.qbase = -1;
            switch (fl.first) {
            case F_TIMESTEP: s.inl_off = 0; break;
            case F_LPA: s.inl_off = 1; break;
            case F_MOMENTS:
                MZ_REQUIRE(p->n_moments == f->n_moments, "mz_nc_props_write: moment count differs from the file");
                s.src = p->moments;
                break;
            case F_NP: s.src = p->np; break;
            case F_NDENS: s.src = p->n; break;
            case F_V: s.src = p->v; break;
            case F_T: s.src = p->T; break;
            default: throw MzError(MZ_E_ARG, "internal: field");
            }
            off += fl.second;
        }
        const int k = acquire_slot(f);
        device_record(f, k, a);
        submit_slot(f, k, true, sync_freq);
        return MZ_OK;
    } catch (MzError& e) {
        report(f, e.what());
        return e.code;
    } catch (std::exception& e) {
        report(f, e.what());
        return MZ_E_ARG;
    }
}

int mz_nc_props_write_host(mz_nc_file* f, const double* lpa, const double* np, const double* ndens, const double* v,
                           const double* T, const double* moments, int32_t ndens_not_Np, double timestep,
                           int32_t sync_freq)
{
    if (!f) return MZ_E_ARG;
    try {
        MZ_REQUIRE(!f->surf, "mz_nc_props_write_host: a surface file");
        MZ_REQUIRE((ndens_not_Np != 0) == (f->ndens_not_Np != 0),
                   "Inconsistent computation of ndens/number of physical particles in cell");
        std::vector<const double*> src;
        for (auto& fl : f->fields) switch (fl.first) {
            case F_TIMESTEP: src.push_back(&timestep); break;
            case F_LPA: src.push_back(lpa); break;
            case F_MOMENTS: src.push_back(moments); break;
            case F_NP: src.push_back(np); break;
            case F_NDENS: src.push_back(ndens); break;
            case F_V: src.push_back(v); break;
            case F_T: src.push_back(T); break;
            default: throw MzError(MZ_E_ARG, "internal: field");
            }
        const int k = acquire_slot(f);
        host_record(f, k, src);
        submit_slot(f, k, false, sync_freq);
        return MZ_OK;
    } catch (MzError& e) {
        report(f, e.what());
        return e.code;
    } catch (std::exception& e) {
        report(f, e.what());
        return MZ_E_ARG;
    }
}

int mz_nc_surf_write(mz_nc_file* f, const mz_surf_props* sp, double timestep, int32_t sync_freq)
{
    if (!f) return MZ_E_ARG;
    try {
        MZ_REQUIRE(f->surf && sp && f->ctx && sp->dom->ctx == f->ctx, "mz_nc_surf_write: bad argument");
        MZ_REQUIRE(sp->dom->ns == f->n_species && f->n_elements == 2, "mz_nc_surf_write: shape differs from the file");
        PackArgs a;
        memset(&a, 0, sizeof a);
        a.inl[0] = timestep;
        int64_t off = 0;
        for (auto& fl : f->fields) {
            PackSeg& s = a.seg[a.nseg++];
            s.n = fl.second;
            s.dst = off;
            s.src = sp->acc;
            s.ncomp = 1;
            // quantity slots of a wall's sums (cell_ops.cuh SurfAcc)
            switch (fl.first) {
            case F_TIMESTEP: s.src = nullptr; s.qbase = -1; s.inl_off = 0; break;
            case F_SNP: s.qbase = 0; break;
            case F_FLUX_IN: s.qbase = 1; break;
            case F_FLUX_OUT: s.qbase = 2; break;
            case F_FORCE: s.qbase = 3; s.ncomp = 3; break;
            case F_PN: s.qbase = 6; break;
            case F_SHEAR: s.qbase = 7; s.ncomp = 3; break;
            case F_KEF: s.qbase = 10; break;
            default: throw MzError(MZ_E_ARG, "internal: field");
            }
            off += fl.second;
        }
        const int k = acquire_slot(f);
        device_record(f, k, a);
        submit_slot(f, k, true, sync_freq);
        return MZ_OK;
    } catch (MzError& e) {
        report(f, e.what());
        return e.code;
    } catch (std::exception& e) {
        report(f, e.what());
        return MZ_E_ARG;
    }
}

int mz_nc_surf_write_host(mz_nc_file* f, const double* np, const double* flux_incident, const double* flux_reflected,
                          const double* force, const double* normal_pressure, const double* shear_pressure,
                          const double* kinetic_energy_flux, double timestep, int32_t sync_freq)
{
    if (!f) return MZ_E_ARG;
    try {
        MZ_REQUIRE(f->surf, "mz_nc_surf_write_host: a cell-property file");
        std::vector<const double*> src;
        for (auto& fl : f->fields) switch (fl.first) {
            case F_TIMESTEP: src.push_back(&timestep); break;
            case F_SNP: src.push_back(np); break;
            case F_FLUX_IN: src.push_back(flux_incident); break;
            case F_FLUX_OUT: src.push_back(flux_reflected); break;
            case F_FORCE: src.push_back(force); break;
            case F_PN: src.push_back(normal_pressure); break;
            case F_SHEAR: src.push_back(shear_pressure); break;
            case F_KEF: src.push_back(kinetic_energy_flux); break;
            default: throw MzError(MZ_E_ARG, "internal: field");
            }
        const int k = acquire_slot(f);
        host_record(f, k, src);
        submit_slot(f, k, false, sync_freq);
        return MZ_OK;
    } catch (MzError& e) {
        report(f, e.what());
        return e.code;
    } catch (std::exception& e) {
        report(f, e.what());
        return MZ_E_ARG;
    }
}

int mz_nc_flush(mz_nc_file* f)
{
    if (!f) return MZ_E_ARG;
    drain(f);
    std::lock_guard<std::mutex> lk(f->m);
    if (!f->io_error.empty()) {
        report(f, f->io_error);
        return MZ_E_ARG;
    }
    return MZ_OK;
}

int mz_nc_records(const mz_nc_file* f, int64_t* n)
{
    if (!f || !n) return MZ_E_ARG;
    *n = f->numrecs;
    return MZ_OK;
}

int mz_nc_close(mz_nc_file* f)
{
    if (!f) return MZ_OK;
    int rc = MZ_OK;
    if (f->th.joinable()) {
        drain(f);
        {
            std::lock_guard<std::mutex> lk(f->m);
            f->stop = true;
        }
        f->cv.notify_all();
        f->th.join();
    }
    if (!f->io_error.empty()) {
        report(f, f->io_error);
        rc = MZ_E_ARG;
    }
    if (f->fd >= 0 && close(f->fd) != 0 && rc == MZ_OK) rc = MZ_E_ARG;
    for (auto& s : f->slot) {
        if (f->ctx) {
            if (s.host) cudaFreeHost(s.host);
            if (s.dev) cudaFree(s.dev);
            if (s.ready) cudaEventDestroy(s.ready);
        } else {
            free(s.host);
        }
    }
    if (f->copy_stream) cudaStreamDestroy(f->copy_stream);
    delete f;
    return rc;
}

int mz_nc_last_error(const mz_nc_file* f, char* buf, size_t len)
{
    if (!f || !buf || len == 0) return MZ_E_ARG;
    snprintf(buf, len, "%s", f->last_error.c_str());
    return MZ_OK;
}

}  // extern "C"
