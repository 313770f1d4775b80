// C ABI of merzgpu (include/merzgpu.h): context, domain storage, particle
// upload/download and dispatch to the kernels in the other translation units.
#include "mz_host.h"

#include <algorithm>
#include <cstdio>
#include <numeric>

using namespace mz;

// ------------------------------------------------------------------ context
cudaEvent_t mz_ctx_s::get_event()
{
    if (!event_pool.empty()) {
        cudaEvent_t e = event_pool.back();
        event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    MZ_CK(cudaEventCreate(&e));
    return e;
}

bool mz_ctx_s::capturing() const
{
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(stream, &st) != cudaSuccess) return false;
    return st == cudaStreamCaptureStatusActive;
}

int mz_ctx_s::timer_begin(const char* name, cudaEvent_t* start)
{
    if (!kernel_timing || capturing()) return -1;
    int slot = -1;
    for (size_t i = 0; i < timings.size(); ++i)
        if (timings[i].name == name) slot = (int)i;
    if (slot < 0) {
        timings.push_back(KernelTiming{});
        timings.back().name = name;
        slot = (int)timings.size() - 1;
    }
    *start = get_event();
    MZ_CK(cudaEventRecord(*start, stream));
    return slot;
}

void mz_ctx_s::timer_end(int slot, cudaEvent_t start)
{
    if (slot < 0) return;
    cudaEvent_t stop = get_event();
    MZ_CK(cudaEventRecord(stop, stream));
    timings[slot].pending.push_back({start, stop});
    timings[slot].launches++;
}

void mz_ctx_s::resolve_timings()
{
    MZ_CK(cudaStreamSynchronize(stream));
    for (auto& t : timings) {
        for (auto& pr : t.pending) {
            float ms = 0.f;
            MZ_CK(cudaEventElapsedTime(&ms, pr.first, pr.second));
            t.total_ms += ms;
            event_pool.push_back(pr.first);
            event_pool.push_back(pr.second);
        }
        t.pending.clear();
    }
}

int64_t div_up(int64_t a, int64_t b) { return (a + b - 1) / b; }

void set_err(const mz_ctx* c, const std::string& m)
{
    if (c) const_cast<mz_ctx*>(c)->last_error = m;
}

// ------------------------------------------------------------------ domain helpers
mz::DomainView make_view(mz_domain* d)
{
    DomainView v;
    memset(&v, 0, sizeof v);
    v.n_cells = (int32_t)d->n_cells;
    v.n_species = d->ns;
    for (int s = 0; s < d->ns; ++s) {
        SpeciesHost& S = d->sp[s];
        SpeciesView& o = v.sp[s];
        o.A = Cols{S.wv[S.cur], S.pos[S.cur]};
        o.B = Cols{S.wv[S.cur ^ 1], S.pos[S.cur ^ 1]};
        o.cell = S.cell[S.cur];
        o.cellB = S.cell[S.cur ^ 1];
        o.key = S.key;
        o.idx = S.idx;
        o.counts = S.counts;
        o.fill = S.fill;
        o.ind = S.ind;
        o.capacity = S.capacity;
        o.mass = d->mass[s];
    }
    for (int i = 0; i < MZ_MAX_SPECIES * MZ_MAX_SPECIES; ++i) v.inter[i] = d->inter[i];
    v.cell_V = d->d_V;
    v.cell_seed = d->d_cell_seed;
    v.cell_rid = d->d_cell_rid;
    v.cell_step = d->d_cell_step;
    v.cf = d->d_cf;
    v.trig = d->ctx->d_trig;
    v.status = d->d_status;
    v.counters = d->d_counters;
    v.seed = d->seed;
    return v;
}

void check_status(mz_domain* d)
{
    int st = 0;
    MZ_CK(cudaMemcpyAsync(&st, d->d_status, sizeof(int), cudaMemcpyDeviceToHost, d->ctx->stream));
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    if (st) {
        int zero = 0;
        MZ_CK(cudaMemcpy(d->d_status, &zero, sizeof(int), cudaMemcpyHostToDevice));
        std::string m = "device status:";
        if (st & ST_CAPACITY) m += " capacity/count limit exceeded or sampled cell not empty;";
        if (st & ST_OUTSIDE_GRID) m += " particle outside the grid;";
        if (st & ST_MERGE_BINS) m += " octree bin limit reached;";
        if (st & ST_SEGMENT) m += " cell too large for the sort path;";
        if (st & ST_WALL_HITS) m += " wall-hit cap reached;";
        if (st & ST_TIMEOUT) m += " a bounded wait for gathered cells gave up;";
        throw MzError((st & ST_TIMEOUT) ? MZ_E_TIMEOUT : MZ_E_STATE, m);
    }
}

static void free_species(SpeciesHost& S)
{
    for (int b = 0; b < 2; ++b) {
        cudaFree(S.wv[b]);
        cudaFree(S.pos[b]);
        cudaFree(S.cell[b]);
    }
    cudaFree(S.key);
    cudaFree(S.idx);
}

static void alloc_cols(SpeciesHost& S, int64_t cap)
{
    for (int b = 0; b < 2; ++b) {
        MZ_CK(cudaMalloc(&S.wv[b], std::max<int64_t>(cap, 1) * sizeof(PV)));
        MZ_CK(cudaMalloc(&S.pos[b], std::max<int64_t>(cap, 1) * sizeof(PX)));
        MZ_CK(cudaMalloc(&S.cell[b], std::max<int64_t>(cap, 1) * sizeof(int32_t)));
    }
    MZ_CK(cudaMalloc(&S.key, std::max<int64_t>(cap, 1) * sizeof(int32_t)));
    MZ_CK(cudaMalloc(&S.idx, std::max<int64_t>(cap, 1) * sizeof(int32_t)));
    S.capacity = cap;
}

void reserve_species(mz_domain* d, int s, int64_t cap)
{
    MZ_REQUIRE(cap < (1ll << 31) - 1024, "reserve: capacity out of range");
    SpeciesHost& S = d->sp[s];
    if (cap <= S.capacity) return;
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    SpeciesHost N;
    alloc_cols(N, cap);
    const int64_t hw = S.hw;
    if (hw > 0) {
        MZ_CK(cudaMemcpyAsync(N.wv[0], S.wv[S.cur], hw * sizeof(PV), cudaMemcpyDeviceToDevice, d->ctx->stream));
        MZ_CK(cudaMemcpyAsync(N.pos[0], S.pos[S.cur], hw * sizeof(PX), cudaMemcpyDeviceToDevice, d->ctx->stream));
        MZ_CK(cudaMemcpyAsync(N.cell[0], S.cell[S.cur], hw * sizeof(int32_t), cudaMemcpyDeviceToDevice, d->ctx->stream));
        MZ_CK(cudaMemcpyAsync(N.key, S.key, hw * sizeof(int32_t), cudaMemcpyDeviceToDevice, d->ctx->stream));
    }
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    free_species(S);
    for (int b = 0; b < 2; ++b) {
        S.wv[b] = N.wv[b];
        S.pos[b] = N.pos[b];
        S.cell[b] = N.cell[b];
    }
    S.key = N.key;
    S.idx = N.idx;
    S.capacity = cap;
    S.cur = 0;
}

// ------------------------------------------------------------------ API
extern "C" {

int mz_version(void) { return MZ_ABI_VERSION; }

int mz_ctx_create(int device, mz_ctx** out)
{
    mz_ctx* c = nullptr;
    API_TRY
    MZ_REQUIRE(out != nullptr, "mz_ctx_create: out is NULL");
    c = new mz_ctx_s();
    c->device = device;
    MZ_CK(cudaSetDevice(device));
    MZ_CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    MZ_CK(cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking));
    MZ_CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
    MZ_CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    MZ_CK(cudaEventCreate(&c->t0));
    MZ_CK(cudaEventCreate(&c->t1));
    MZ_CK(cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device));
    {
        // {sin, cos} at the sector centres 2 pi (i + 1/2) / TRIG_SECTORS in
        // extended precision, split into leading and trailing doubles
        std::vector<double2> tab(2 * mz::TRIG_SECTORS);
        const long double pi = acosl(-1.0L);
        for (int i = 0; i < mz::TRIG_SECTORS; ++i) {
            const long double a = 2.0L * pi * ((long double)i + 0.5L) / (long double)mz::TRIG_SECTORS;
            const long double sa = sinl(a), ca = cosl(a);
            const double sh = (double)sa, ch = (double)ca;
            tab[2 * i] = make_double2(sh, ch);
            tab[2 * i + 1] = make_double2((double)(sa - (long double)sh), (double)(ca - (long double)ch));
        }
        MZ_CK(cudaMalloc(&c->d_trig, tab.size() * sizeof(double2)));
        MZ_CK(cudaMemcpy(c->d_trig, tab.data(), tab.size() * sizeof(double2), cudaMemcpyHostToDevice));
    }
    *out = c;
    API_CATCH(c)
}

int mz_ctx_destroy(mz_ctx* c)
{
    if (!c) return MZ_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    for (auto& t : c->timings)
        for (auto& p : t.pending) {
            cudaEventDestroy(p.first);
            cudaEventDestroy(p.second);
        }
    for (auto e : c->event_pool) cudaEventDestroy(e);
    if (c->t0) cudaEventDestroy(c->t0);
    if (c->t1) cudaEventDestroy(c->t1);
    if (c->flush_buf) cudaFree(c->flush_buf);
    if (c->d_trig) cudaFree(c->d_trig);
    if (c->side) {
        cudaStreamSynchronize(c->side);
        cudaStreamDestroy(c->side);
    }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    cudaStreamDestroy(c->stream);
    delete c;
    return MZ_OK;
}

int mz_ctx_synchronize(mz_ctx* c)
{
    API_TRY
    MZ_REQUIRE(c, "NULL context");
    MZ_CK(cudaSetDevice(c->device));
    MZ_CK(cudaStreamSynchronize(c->stream));
    API_CATCH(c)
}

int mz_last_error(const mz_ctx* c, char* buf, size_t len)
{
    if (!c || !buf || len == 0) return MZ_E_ARG;
    snprintf(buf, len, "%s", c->last_error.c_str());
    return MZ_OK;
}

int mz_ctx_stream(mz_ctx* c, void** stream)
{
    if (!c || !stream) return MZ_E_ARG;
    *stream = (void*)c->stream;
    return MZ_OK;
}

int mz_timer_start(mz_ctx* c)
{
    API_TRY
    MZ_REQUIRE(c, "NULL context");
    MZ_CK(cudaEventRecord(c->t0, c->stream));
    API_CATCH(c)
}

int mz_timer_stop(mz_ctx* c, double* ms)
{
    API_TRY
    MZ_REQUIRE(c && ms, "NULL argument");
    MZ_CK(cudaEventRecord(c->t1, c->stream));
    MZ_CK(cudaEventSynchronize(c->t1));
    float f = 0.f;
    MZ_CK(cudaEventElapsedTime(&f, c->t0, c->t1));
    *ms = f;
    API_CATCH(c)
}

int mz_ctx_flush_l2(mz_ctx* c)
{
    API_TRY
    MZ_REQUIRE(c, "NULL context");
    if (!c->flush_buf) {
        c->flush_bytes = (size_t)512 << 20;
        MZ_CK(cudaMalloc(&c->flush_buf, c->flush_bytes));
    }
    MZ_CK(cudaMemsetAsync(c->flush_buf, (int)(c->launches & 0xFF), c->flush_bytes, c->stream));
    API_CATCH(c)
}

int mz_ctx_set_kernel_timing(mz_ctx* c, int enable)
{
    API_TRY
    MZ_REQUIRE(c, "NULL context");
    c->resolve_timings();
    c->kernel_timing = enable != 0;
    if (enable)
        for (auto& t : c->timings) {
            t.total_ms = 0.0;
            t.launches = 0;
        }
    API_CATCH(c)
}

int mz_kernel_timing(mz_ctx* c, int k, char* name, size_t len, double* total_ms, int64_t* launches, int* n_kernels)
{
    API_TRY
    MZ_REQUIRE(c, "NULL context");
    c->resolve_timings();
    if (n_kernels) *n_kernels = (int)c->timings.size();
    if (k >= 0 && k < (int)c->timings.size()) {
        if (name && len) snprintf(name, len, "%s", c->timings[k].name.c_str());
        if (total_ms) *total_ms = c->timings[k].total_ms;
        if (launches) *launches = c->timings[k].launches;
    }
    API_CATCH(c)
}

int mz_launch_count(mz_ctx* c, int64_t* launches)
{
    if (!c || !launches) return MZ_E_ARG;
    *launches = c->launches;
    return MZ_OK;
}

int mz_domain_create(mz_ctx* c, int64_t n_cells, int32_t n_species, const int64_t* capacity, mz_domain** out)
{
    mz_domain* d = nullptr;
    API_TRY
    MZ_REQUIRE(c && out && capacity, "mz_domain_create: NULL argument");
    MZ_REQUIRE(n_cells >= 1 && n_cells < (1ll << 30), "mz_domain_create: n_cells out of range");
    MZ_REQUIRE(n_species >= 1 && n_species <= MZ_MAX_SPECIES, "mz_domain_create: n_species must be 1..4");
    MZ_CK(cudaSetDevice(c->device));
    d = new mz_domain_s();
    d->ctx = c;
    d->n_cells = n_cells;
    d->ns = n_species;
    memset(d->inter, 0, sizeof d->inter);
    for (int s = 0; s < n_species; ++s) {
        MZ_REQUIRE(capacity[s] >= 0 && capacity[s] < (1ll << 31) - 1024, "mz_domain_create: capacity out of range");
        SpeciesHost& S = d->sp[s];
        alloc_cols(S, capacity[s]);
        MZ_CK(cudaMalloc(&S.counts, (n_cells + 1) * sizeof(int32_t)));
        MZ_CK(cudaMalloc(&S.fill, (n_cells + 1) * sizeof(int32_t)));
        MZ_CK(cudaMalloc(&S.work, (n_cells + 1) * sizeof(int32_t)));
        MZ_CK(cudaMalloc(&S.ind, n_cells * sizeof(Indexer)));
        MZ_CK(cudaMemset(S.counts, 0, (n_cells + 1) * sizeof(int32_t)));
        MZ_CK(cudaMemset(S.fill, 0, (n_cells + 1) * sizeof(int32_t)));
        MZ_CK(cudaMemset(S.ind, 0, n_cells * sizeof(Indexer)));
    }
    MZ_CK(cudaMalloc(&d->d_V, n_cells * sizeof(double)));
    std::vector<double> ones(n_cells, 1.0);
    MZ_CK(cudaMemcpy(d->d_V, ones.data(), n_cells * sizeof(double), cudaMemcpyHostToDevice));
    const size_t ncf = (size_t)n_species * n_species * n_cells;
    MZ_CK(cudaMalloc(&d->d_cf, ncf * sizeof(CollisionFactors)));
    MZ_CK(cudaMemset(d->d_cf, 0, ncf * sizeof(CollisionFactors)));
    MZ_CK(cudaMalloc(&d->d_counters, sizeof(Counters)));
    MZ_CK(cudaMemset(d->d_counters, 0, sizeof(Counters)));
    MZ_CK(cudaMalloc(&d->d_status, sizeof(int)));
    MZ_CK(cudaMemset(d->d_status, 0, sizeof(int)));
    MZ_CK(cudaMalloc(&d->d_scalar, 16 * sizeof(int64_t)));
    MZ_CK(cudaMalloc(&d->d_tile_sums, (scan_tiles(n_cells) + 1) * sizeof(int64_t)));
    MZ_CK(cudaMallocHost(&d->h_scalar, 8 * sizeof(int64_t)));
    *out = d;
    d = nullptr;
    API_CATCH(c)
}

static void free_props(mz_props* p)
{
    free_props_snapshot(p);
    cudaFree(p->np);
    cudaFree(p->n);
    cudaFree(p->v);
    cudaFree(p->T);
    cudaFree(p->moments);
    delete p;
}

int mz_domain_destroy(mz_domain* d)
{
    if (!d) return MZ_OK;
    cudaSetDevice(d->ctx->device);
    cudaStreamSynchronize(d->ctx->stream);
    for (mz_props* p : d->props) free_props(p);
    d->props.clear();
    for (mz_surf_props* p : d->surf) {
        cudaFree(p->acc);
        delete p;
    }
    d->surf.clear();
    for (int s = 0; s < d->ns; ++s) {
        free_species(d->sp[s]);
        cudaFree(d->sp[s].counts);
        cudaFree(d->sp[s].fill);
        cudaFree(d->sp[s].work);
        cudaFree(d->sp[s].ind);
    }
    cudaFree(d->d_V);
    cudaFree(d->d_cell_seed);
    cudaFree(d->d_cell_rid);
    cudaFree(d->d_cell_step);
    cudaFree(d->d_cf);
    cudaFree(d->d_counters);
    cudaFree(d->d_status);
    cudaFree(d->d_scalar);
    cudaFree(d->d_tile_sums);
    cudaFree(d->d_merge_scratch);
    cudaFree(d->d_step);
    cudaFree(d->d_done);
    cudaFree(d->d_hitq);
    cudaFree(d->d_vw);
    cudaFreeHost(d->h_vw);
    cudaFree(d->d_ready);
    free_slab_scratch(d);
    cudaFreeHost(d->h_scalar);
    delete d;
    return MZ_OK;
}

int mz_domain_reserve(mz_domain* d, int32_t s, int64_t cap)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns, "mz_domain_reserve: bad species");
    MZ_CK(cudaSetDevice(d->ctx->device));
    reserve_species(d, s, cap);
    API_CATCH(d->ctx)
}

int mz_domain_info(mz_domain* d, int32_t s, int64_t* capacity, int64_t* n_total, int64_t* high_water)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns, "mz_domain_info: bad species");
    check_status(d);
    if (capacity) *capacity = d->sp[s].capacity;
    if (n_total) *n_total = d->sp[s].n_total;
    if (high_water) *high_water = d->sp[s].hw;
    API_CATCH(d->ctx)
}

int mz_set_species(mz_domain* d, const double* mass)
{
    API_TRY
    MZ_REQUIRE(d && mass, "mz_set_species: NULL argument");
    for (int s = 0; s < d->ns; ++s) {
        MZ_REQUIRE(mass[s] > 0.0, "mz_set_species: mass must be positive");
        d->mass[s] = mass[s];
    }
    API_CATCH(d->ctx)
}

int mz_set_interactions(mz_domain* d, const mz_interaction* inter)
{
    API_TRY
    MZ_REQUIRE(d && inter, "mz_set_interactions: NULL argument");
    for (int i = 0; i < d->ns * d->ns; ++i) {
        const mz_interaction& a = inter[i];
        const int s1 = i % d->ns, s2 = i / d->ns;
        d->inter[s1 + d->ns * s2] =
            Interaction{a.m_r, a.mu1, a.mu2, a.vhs_d, a.vhs_o, a.vhs_Tref, a.vhs_muref, a.vhs_factor};
    }
    API_CATCH(d->ctx)
}

int mz_set_cell_volumes(mz_domain* d, const double* V)
{
    API_TRY
    MZ_REQUIRE(d, "NULL domain");
    std::vector<double> v(d->n_cells, 1.0);
    if (V)
        for (int64_t i = 0; i < d->n_cells; ++i) {
            MZ_REQUIRE(V[i] > 0.0, "mz_set_cell_volumes: volumes must be positive");
            v[i] = V[i];
        }
    MZ_CK(cudaMemcpy(d->d_V, v.data(), d->n_cells * sizeof(double), cudaMemcpyHostToDevice));
    API_CATCH(d->ctx)
}

int mz_set_seed(mz_domain* d, uint64_t seed)
{
    if (!d) return MZ_E_ARG;
    d->seed = seed;
    return MZ_OK;
}

int mz_set_cell_rng(mz_domain* d, const uint64_t* seed, const uint32_t* rid, const uint32_t* step_offset)
{
    API_TRY
    MZ_REQUIRE(d, "NULL domain");
    const int64_t n = d->n_cells;
    auto put = [&](auto** dst, const auto* src, size_t esz) {
        if (!src) {
            cudaFree(*dst);
            *dst = nullptr;
            return;
        }
        if (!*dst) MZ_CK(cudaMalloc((void**)dst, n * esz));
        MZ_CK(cudaMemcpy(*dst, src, n * esz, cudaMemcpyHostToDevice));
    };
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    put(&d->d_cell_seed, seed, sizeof(uint64_t));
    put(&d->d_cell_rid, rid, sizeof(uint32_t));
    put(&d->d_cell_step, step_offset, sizeof(uint32_t));
    API_CATCH(d->ctx)
}

namespace {
// records from the caller's columns staged in device memory
__global__ void k_pack(int64_t n, const double* w, const double* v, const double* x, PV* ov, PX* ox)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        ov[i] = PV{w[i], v[3 * i], v[3 * i + 1], v[3 * i + 2]};
        ox[i] = PX{x[3 * i], x[3 * i + 1], x[3 * i + 2], 0.0};
    }
}
}  // namespace

// w (n), v (3n) and x (3n, row-major) into buffer A's records: the columns
// are staged in buffer B (free outside a sort) and packed on the device
static void upload_cols(mz_domain* d, int s, int64_t n, const double* w, const double* v, const double* x)
{
    SpeciesHost& S = d->sp[s];
    mz_ctx* c = d->ctx;
    double* sw = reinterpret_cast<double*>(S.wv[S.cur ^ 1]);  // 4n doubles: w then v
    double* sv = sw + n;
    double* sx = reinterpret_cast<double*>(S.pos[S.cur ^ 1]);  // 3n doubles
    MZ_CK(cudaMemcpyAsync(sw, w, n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(sv, v, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(sx, x, 3 * n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(n, 256), (int64_t)c->num_sms * 8));
    MZ_LAUNCH(c, "pack", k_pack, blocks, 256, 0, n, sw, sv, sx, S.wv[S.cur], S.pos[S.cur]);
    MZ_CK(cudaStreamSynchronize(c->stream));
}

int mz_upload_particles(mz_domain* d, int32_t s, int64_t n, const double* w, const double* v, const double* x,
                        const int32_t* cell)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns, "mz_upload_particles: bad species");
    MZ_REQUIRE(n >= 0 && (n == 0 || (w && v && x && cell)), "mz_upload_particles: NULL data");
    MZ_CK(cudaSetDevice(d->ctx->device));
    for (int64_t i = 0; i < n; ++i)
        MZ_REQUIRE(cell[i] >= 0 && cell[i] < d->n_cells, "mz_upload_particles: cell id out of range");
    if (n > d->sp[s].capacity) {
        d->sp[s].hw = 0;
        reserve_species(d, s, n);
    }
    SpeciesHost& S = d->sp[s];
    if (n > 0) {
        upload_cols(d, s, n, w, v, x);
        MZ_CK(cudaMemcpy(S.cell[S.cur], cell, n * sizeof(int32_t), cudaMemcpyHostToDevice));
        MZ_CK(cudaMemcpy(S.key, cell, n * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    S.hw = n;
    S.n_total = n;
    launch_sort(d, s, nullptr, nullptr);
    check_status(d);
    API_CATCH(d->ctx)
}

int mz_upload_particles_indexed(mz_domain* d, int32_t s, int64_t n_slots, const double* w, const double* v,
                                const double* x, const mz_particle_indexer* ind)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns && ind, "mz_upload_particles_indexed: bad argument");
    MZ_REQUIRE(n_slots >= 0 && (n_slots == 0 || (w && v && x)), "mz_upload_particles_indexed: NULL data");
    MZ_CK(cudaSetDevice(d->ctx->device));
    std::vector<int32_t> owner(n_slots, -1);
    std::vector<Indexer> di(d->n_cells);
    int64_t total = 0;
    for (int64_t c = 0; c < d->n_cells; ++c) {
        const mz_particle_indexer& p = ind[c];
        MZ_REQUIRE(p.n_group1 >= 0 && p.n_group2 >= 0 && p.n_local == p.n_group1 + p.n_group2,
                   "mz_upload_particles_indexed: inconsistent indexer");
        auto mark = [&](int64_t st, int64_t n) {
            MZ_REQUIRE(n == 0 || (st >= 0 && st + n <= n_slots), "mz_upload_particles_indexed: group out of range");
            for (int64_t i = st; i < st + n; ++i) {
                MZ_REQUIRE(owner[i] < 0, "mz_upload_particles_indexed: overlapping groups");
                owner[i] = (int32_t)c;
            }
        };
        mark(p.start1, p.n_group1);
        mark(p.start2, p.n_group2);
        di[c] = Indexer{p.n_group1 ? (int32_t)p.start1 : 0, (int32_t)p.n_group1, p.n_group2 ? (int32_t)p.start2 : 0,
                        (int32_t)p.n_group2};
        total += p.n_local;
    }
    if (n_slots > d->sp[s].capacity) {
        d->sp[s].hw = 0;
        reserve_species(d, s, n_slots);
    }
    SpeciesHost& S = d->sp[s];
    if (n_slots > 0) {
        upload_cols(d, s, n_slots, w, v, x);
        MZ_CK(cudaMemcpy(S.cell[S.cur], owner.data(), n_slots * sizeof(int32_t), cudaMemcpyHostToDevice));
        MZ_CK(cudaMemcpy(S.key, owner.data(), n_slots * sizeof(int32_t), cudaMemcpyHostToDevice));
    }
    MZ_CK(cudaMemcpy(S.ind, di.data(), d->n_cells * sizeof(Indexer), cudaMemcpyHostToDevice));
    S.hw = n_slots;
    S.n_total = total;
    S.compact = false;
    S.group2 = true;
    API_CATCH(d->ctx)
}

int mz_download_particles(mz_domain* d, int32_t s, int64_t max_n, double* w, double* v, double* x, int32_t* cell,
                          int64_t* n_out)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns, "mz_download_particles: bad species");
    MZ_CK(cudaSetDevice(d->ctx->device));
    check_status(d);
    SpeciesHost& S = d->sp[s];
    const int64_t hw = S.hw;
    std::vector<Indexer> ind(d->n_cells);
    MZ_CK(cudaMemcpy(ind.data(), S.ind, d->n_cells * sizeof(Indexer), cudaMemcpyDeviceToHost));
    int64_t total = 0;
    for (auto& p : ind) total += p.n1 + p.n2;
    if (n_out) *n_out = total;
    if (total > max_n) throw MzError(MZ_E_CAPACITY, "mz_download_particles: output buffers too small");
    std::vector<PV> rv(std::max<int64_t>(hw, 1));
    std::vector<PX> rx(std::max<int64_t>(hw, 1));
    if (hw > 0) {
        MZ_CK(cudaMemcpy(rv.data(), S.wv[S.cur], hw * sizeof(PV), cudaMemcpyDeviceToHost));
        MZ_CK(cudaMemcpy(rx.data(), S.pos[S.cur], hw * sizeof(PX), cudaMemcpyDeviceToHost));
    }
    int64_t o = 0;
    for (int64_t c = 0; c < d->n_cells; ++c) {
        const Indexer p = ind[c];
        for (int32_t j = 0; j < p.n1 + p.n2; ++j, ++o) {
            const int64_t q = j < p.n1 ? p.start1 + j : p.start2 + (j - p.n1);
            MZ_REQUIRE(q >= 0 && q < hw, "mz_download_particles: indexer points outside the slots in use");
            if (w) w[o] = rv[q].w;
            if (v) {
                v[3 * o] = rv[q].vx;
                v[3 * o + 1] = rv[q].vy;
                v[3 * o + 2] = rv[q].vz;
            }
            if (x) {
                x[3 * o] = rx[q].x;
                x[3 * o + 1] = rx[q].y;
                x[3 * o + 2] = rx[q].z;
            }
            if (cell) cell[o] = (int32_t)c;
        }
    }
    API_CATCH(d->ctx)
}

int mz_get_indexer(mz_domain* d, int32_t s, mz_particle_indexer* out, int64_t* n_total)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns, "mz_get_indexer: bad species");
    MZ_CK(cudaSetDevice(d->ctx->device));
    check_status(d);
    std::vector<Indexer> ind(d->n_cells);
    MZ_CK(cudaMemcpy(ind.data(), d->sp[s].ind, d->n_cells * sizeof(Indexer), cudaMemcpyDeviceToHost));
    int64_t tot = 0;
    for (int64_t c = 0; c < d->n_cells; ++c) {
        const Indexer p = ind[c];
        tot += p.n1 + p.n2;
        if (out) {
            mz_particle_indexer& q = out[c];
            q.n_local = p.n1 + p.n2;
            q.n_group1 = p.n1;
            q.start1 = p.n1 ? p.start1 : 0;
            q.end1 = p.n1 ? (int64_t)p.start1 + p.n1 - 1 : -1;
            q.n_group2 = p.n2;
            q.start2 = p.n2 ? p.start2 : 0;
            q.end2 = p.n2 ? (int64_t)p.start2 + p.n2 - 1 : -1;
        }
    }
    if (n_total) *n_total = tot;
    API_CATCH(d->ctx)
}

int mz_set_collision_factors(mz_domain* d, int32_t s1, int32_t s2, const double* smax)
{
    API_TRY
    MZ_REQUIRE(d && smax && s1 >= 0 && s2 >= 0 && s1 < d->ns && s2 < d->ns, "mz_set_collision_factors: bad argument");
    MZ_CK(cudaSetDevice(d->ctx->device));
    const int64_t nc = d->n_cells;
    CollisionFactors* base = d->d_cf + (size_t)(s1 + d->ns * s2) * nc;
    std::vector<CollisionFactors> cf(nc);
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    MZ_CK(cudaMemcpy(cf.data(), base, nc * sizeof(CollisionFactors), cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < nc; ++c) cf[c].smax = smax[c];
    MZ_CK(cudaMemcpy(base, cf.data(), nc * sizeof(CollisionFactors), cudaMemcpyHostToDevice));
    API_CATCH(d->ctx)
}

int mz_get_collision_factors(mz_domain* d, int32_t s1, int32_t s2, mz_collision_factors* out)
{
    API_TRY
    MZ_REQUIRE(d && out && s1 >= 0 && s2 >= 0 && s1 < d->ns && s2 < d->ns, "mz_get_collision_factors: bad argument");
    MZ_CK(cudaSetDevice(d->ctx->device));
    check_status(d);
    const int64_t nc = d->n_cells;
    std::vector<CollisionFactors> cf(nc);
    MZ_CK(cudaMemcpy(cf.data(), d->d_cf + (size_t)(s1 + d->ns * s2) * nc, nc * sizeof(CollisionFactors),
                     cudaMemcpyDeviceToHost));
    for (int64_t c = 0; c < nc; ++c) {
        out[c].n1 = cf[c].n1;
        out[c].n2 = cf[c].n2;
        out[c].sigma_g_w_max = cf[c].smax;
        out[c].n_coll = cf[c].n_coll;
        out[c].n_coll_performed = cf[c].n_coll_performed;
        out[c].n_eq_w_coll_performed = cf[c].n_eq_w_coll_performed;
    }
    API_CATCH(d->ctx)
}

int mz_ntc(mz_domain* d, int32_t s1, int32_t s2, double dt, int64_t cb, int64_t ce, uint64_t step, int32_t flags,
           double dw_tol)
{
    API_TRY
    MZ_REQUIRE(d && s1 >= 0 && s2 >= 0 && s1 < d->ns && s2 < d->ns, "mz_ntc: bad species");
    MZ_REQUIRE(cb >= 0 && ce <= d->n_cells && cb <= ce, "mz_ntc: bad cell range");
    MZ_CK(cudaSetDevice(d->ctx->device));
    if (cb == ce) return MZ_OK;
    launch_ntc(d, s1, s2, dt, cb, ce, step, flags, dw_tol);
    API_CATCH(d->ctx)
}

int mz_props_create(mz_domain* d, int32_t n_moments, const int32_t* powers, double Tref, int32_t ndens, mz_props** out)
{
    mz_props* p = nullptr;
    API_TRY
    MZ_REQUIRE(d && out && n_moments >= 0 && n_moments <= 16 && (n_moments == 0 || powers),
               "mz_props_create: bad argument");
    MZ_CK(cudaSetDevice(d->ctx->device));
    p = new mz_props_s();
    p->dom = d;
    p->n_moments = n_moments;
    for (int i = 0; i < n_moments; ++i) p->powers[i] = powers[i];
    p->Tref = Tref;
    p->ndens = ndens;
    const size_t m = (size_t)d->n_cells * d->ns;
    MZ_CK(cudaMalloc(&p->np, m * sizeof(double)));
    MZ_CK(cudaMalloc(&p->n, m * sizeof(double)));
    MZ_CK(cudaMalloc(&p->v, 3 * m * sizeof(double)));
    MZ_CK(cudaMalloc(&p->T, m * sizeof(double)));
    MZ_CK(cudaMalloc(&p->moments, std::max<size_t>(1, n_moments * m) * sizeof(double)));
    d->props.push_back(p);
    *out = p;
    int r = mz_clear_props(p);
    p = nullptr;
    if (r) return r;
    API_CATCH(d->ctx)
}

int mz_props_destroy(mz_props* p)
{
    if (!p) return MZ_OK;
    mz_domain* d = p->dom;
    cudaSetDevice(d->ctx->device);
    cudaStreamSynchronize(d->ctx->stream);
    d->props.erase(std::remove(d->props.begin(), d->props.end(), p), d->props.end());
    free_props(p);
    return MZ_OK;
}

int mz_compute_props(mz_domain* d, mz_props* p, int32_t mode)
{
    API_TRY
    MZ_REQUIRE(d && p && p->dom == d, "mz_compute_props: bad argument");
    MZ_REQUIRE(mode >= 0 && mode <= 2, "mz_compute_props: bad mode");
    MZ_CK(cudaSetDevice(d->ctx->device));
    launch_props(d, p, mode);
    API_CATCH(d->ctx)
}

int mz_avg_props(mz_props* avg, const mz_props* inst, double n_avg)
{
    API_TRY
    MZ_REQUIRE(avg && inst && avg->dom == inst->dom, "mz_avg_props: bad argument");
    if (avg->ndens != inst->ndens)
        throw MzError(MZ_E_ARG, "Inconsistent computation of ndens/number of physical particles in cell");
    mz_domain* d = avg->dom;
    MZ_CK(cudaSetDevice(d->ctx->device));
    const int64_t m = d->n_cells * d->ns;
    const double inv = 1.0 / n_avg;
    launch_avg(d->ctx, avg->np, inst->np, m, inv);
    launch_avg(d->ctx, avg->n, inst->n, m, inv);
    launch_avg(d->ctx, avg->v, inst->v, 3 * m, inv);
    launch_avg(d->ctx, avg->T, inst->T, m, inv);
    for (int s = 0; s < d->ns; ++s) avg->lpa[s] = std::fma(inst->lpa[s], inv, avg->lpa[s]);
    API_CATCH(avg ? avg->dom->ctx : nullptr)
}

int mz_clear_props(mz_props* p)
{
    API_TRY
    MZ_REQUIRE(p, "NULL props");
    mz_domain* d = p->dom;
    const size_t m = (size_t)d->n_cells * d->ns;
    cudaStream_t st = d->ctx->stream;
    MZ_CK(cudaMemsetAsync(p->np, 0, m * sizeof(double), st));
    MZ_CK(cudaMemsetAsync(p->n, 0, m * sizeof(double), st));
    MZ_CK(cudaMemsetAsync(p->v, 0, 3 * m * sizeof(double), st));
    MZ_CK(cudaMemsetAsync(p->T, 0, m * sizeof(double), st));
    MZ_CK(cudaMemsetAsync(p->moments, 0, std::max<size_t>(1, p->n_moments * m) * sizeof(double), st));
    for (int s = 0; s < MZ_MAX_SPECIES; ++s) p->lpa[s] = 0.0;
    API_CATCH(p ? p->dom->ctx : nullptr)
}

int mz_props_download(mz_props* p, double* lpa, double* np, double* n, double* v, double* T, double* moments)
{
    API_TRY
    MZ_REQUIRE(p, "NULL props");
    mz_domain* d = p->dom;
    MZ_CK(cudaSetDevice(d->ctx->device));
    check_status(d);
    const size_t m = (size_t)d->n_cells * d->ns;
    if (lpa)
        for (int s = 0; s < d->ns; ++s) lpa[s] = p->lpa[s];
    if (np) MZ_CK(cudaMemcpy(np, p->np, m * sizeof(double), cudaMemcpyDeviceToHost));
    if (n) MZ_CK(cudaMemcpy(n, p->n, m * sizeof(double), cudaMemcpyDeviceToHost));
    if (v) MZ_CK(cudaMemcpy(v, p->v, 3 * m * sizeof(double), cudaMemcpyDeviceToHost));
    if (T) MZ_CK(cudaMemcpy(T, p->T, m * sizeof(double), cudaMemcpyDeviceToHost));
    if (moments && p->n_moments)
        MZ_CK(cudaMemcpy(moments, p->moments, p->n_moments * m * sizeof(double), cudaMemcpyDeviceToHost));
    API_CATCH(p ? p->dom->ctx : nullptr)
}

int mz_convect_1d(mz_domain* d, int32_t s, const mz_grid1d* g, const mz_walls1d* w, double dt, uint64_t step,
                  int32_t flags)
{
    API_TRY
    MZ_REQUIRE(d && g && w && s >= 0 && s < d->ns, "mz_convect_1d: bad argument");
    // a slab of a larger grid convects on the global grid and walls without
    // computing cells (mz_slab_extract maps positions to cells afterwards)
    MZ_REQUIRE(g->n_cells == d->n_cells || (!(flags & MZ_CONVECT_COMPUTE_CELL) && g->n_cells > d->n_cells),
               "mz_convect_1d: grid and domain cell counts differ");
    MZ_CK(cudaSetDevice(d->ctx->device));
    launch_convect(d, s, g, w, dt, step, flags);
    API_CATCH(d->ctx)
}

int mz_sort(mz_domain* d, int32_t s, const mz_grid1d* g, int64_t* out_index)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns, "mz_sort: bad species");
    MZ_REQUIRE(!g || g->n_cells == d->n_cells, "mz_sort: grid and domain cell counts differ");
    MZ_CK(cudaSetDevice(d->ctx->device));
    launch_sort(d, s, g, out_index);
    check_status(d);
    API_CATCH(d->ctx)
}

int mz_squash(mz_domain* d, int32_t s)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns, "mz_squash: bad species");
    MZ_CK(cudaSetDevice(d->ctx->device));
    launch_compact(d, s);
    API_CATCH(d->ctx)
}

int mz_merge_octree_n2(mz_domain* d, int32_t s, int64_t cb, int64_t ce, int64_t threshold, int64_t target,
                       const mz_octree_params* prm, const mz_grid1d* g, uint64_t step, int64_t* n_merged)
{
    API_TRY
    MZ_REQUIRE(d && prm && s >= 0 && s < d->ns, "mz_merge_octree_n2: bad argument");
    MZ_REQUIRE(cb >= 0 && ce <= d->n_cells && cb <= ce, "mz_merge_octree_n2: bad cell range");
    MZ_REQUIRE(target >= 2, "mz_merge_octree_n2: target_np must be >= 2");
    MZ_REQUIRE(!g || g->n_cells == d->n_cells, "mz_merge_octree_n2: grid and domain cell counts differ");
    MZ_CK(cudaSetDevice(d->ctx->device));
    launch_merge(d, s, cb, ce, threshold, target, prm, g, step, n_merged);
    API_CATCH(d->ctx)
}

int mz_sample_cells(mz_domain* d, int32_t s, const int64_t* counts, const double* T3, const double* T3_all,
                    const double* Fnum, double span, const double* box6, int32_t distribution, uint64_t step,
                    const double* v0, const double* v0_all)
{
    API_TRY
    MZ_REQUIRE(d && counts && Fnum && s >= 0 && s < d->ns, "mz_sample_cells: bad argument");
    MZ_REQUIRE(T3 || T3_all, "mz_sample_cells: temperatures missing");
    MZ_REQUIRE(distribution == 0 || distribution == 1, "mz_sample_cells: distribution must be 0 or 1");
    MZ_REQUIRE(d->mass[s] > 0.0, "mz_sample_cells: species mass not set");
    MZ_CK(cudaSetDevice(d->ctx->device));
    launch_sample_cells(d, s, counts, nullptr, T3, T3_all, Fnum, span, box6, distribution, step, v0, v0_all);
    check_status(d);
    API_CATCH(d->ctx)
}

int mz_sample_grid_ndens(mz_domain* d, int32_t s, const mz_grid1d* g, double ndens, double T, double Fnum,
                         uint64_t step, const double* v0)
{
    API_TRY
    MZ_REQUIRE(d && g && s >= 0 && s < d->ns && Fnum > 0.0, "mz_sample_grid_ndens: bad argument");
    MZ_REQUIRE(g->n_cells == d->n_cells, "mz_sample_grid_ndens: grid and domain cell counts differ");
    MZ_REQUIRE(d->mass[s] > 0.0, "mz_sample_grid_ndens: species mass not set");
    MZ_CK(cudaSetDevice(d->ctx->device));
    launch_sample_grid(d, s, g, ndens, T, Fnum, step, v0);
    check_status(d);
    API_CATCH(d->ctx)
}

int mz_step(mz_domain* d, const mz_step_plan* plan, int64_t n_steps, mz_props* inst, mz_props* avg)
{
    API_TRY
    MZ_REQUIRE(d && plan && n_steps >= 0, "mz_step: bad argument");
    MZ_REQUIRE(plan->dims == 0 || plan->dims == 1, "mz_step: dims must be 0 or 1");
    MZ_REQUIRE(!inst || inst->dom == d, "mz_step: props of another domain");
    MZ_REQUIRE(!avg || avg->dom == d, "mz_step: props of another domain");
    MZ_REQUIRE(plan->dims == 0 || plan->grid.n_cells == d->n_cells, "mz_step: grid and domain cell counts differ");
    MZ_CK(cudaSetDevice(d->ctx->device));
    launch_step(d, plan, n_steps, inst, avg);
    API_CATCH(d->ctx)
}

int mz_step_autotune(mz_domain* d, const mz_step_plan* plan, int64_t trial_steps, int32_t* lanes, int32_t* big_cell)
{
    API_TRY
    MZ_REQUIRE(d && plan, "mz_step_autotune: NULL argument");
    MZ_REQUIRE(trial_steps >= 1, "mz_step_autotune: trial_steps must be >= 1");
    MZ_REQUIRE(plan->dims == 0 || plan->dims == 1, "mz_step_autotune: dims must be 0 or 1");
    MZ_CK(cudaSetDevice(d->ctx->device));
    autotune_step(d, plan, trial_steps, lanes, big_cell);
    check_status(d);
    API_CATCH(d->ctx)
}

int mz_get_counters(mz_domain* d, mz_counters* out, int32_t reset)
{
    API_TRY
    MZ_REQUIRE(d && out, "mz_get_counters: bad argument");
    MZ_CK(cudaSetDevice(d->ctx->device));
    Counters c;
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    MZ_CK(cudaMemcpy(&c, d->d_counters, sizeof c, cudaMemcpyDeviceToHost));
    out->candidates = c.candidates;
    out->accepted = c.accepted;
    out->splits = c.splits;
    out->merges = c.merges;
    out->wall_hits = c.wall_hits;
    if (reset) MZ_CK(cudaMemset(d->d_counters, 0, sizeof(Counters)));
    API_CATCH(d->ctx)
}

}  // extern "C"

namespace {
__global__ void k_sincos_2pi(const double2* tab, int64_t n, const uint64_t* m, double* s, double* c)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double a, b;
        mz::sincos_2pi_u52(tab, m[i] & 0xFFFFFFFFFFFFFull, a, b);
        s[i] = a;
        c[i] = b;
    }
}
}  // namespace

int mz_sincos_2pi(mz_ctx* c, int64_t n, const uint64_t* m, double* s, double* co)
{
    struct DevBuf {
        void* p = nullptr;
        ~DevBuf() { if (p) cudaFree(p); }
    };
    API_TRY
    MZ_REQUIRE(c && n >= 0 && (n == 0 || (m && s && co)), "mz_sincos_2pi: bad arguments");
    if (n == 0) return MZ_OK;
    MZ_CK(cudaSetDevice(c->device));
    DevBuf dm, ds;
    MZ_CK(cudaMalloc(&dm.p, n * sizeof(uint64_t)));
    MZ_CK(cudaMalloc(&ds.p, 2 * n * sizeof(double)));
    uint64_t* um = static_cast<uint64_t*>(dm.p);
    double* out = static_cast<double*>(ds.p);
    MZ_CK(cudaMemcpyAsync(um, m, n * sizeof(uint64_t), cudaMemcpyHostToDevice, c->stream));
    const int blocks = (int)std::min<int64_t>(div_up(n, 256), 4096);
    MZ_LAUNCH(c, "sincos_2pi", k_sincos_2pi, blocks, 256, 0, c->d_trig, n, um, out, out + n);
    MZ_CK(cudaMemcpyAsync(s, out, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaMemcpyAsync(co, out + n, n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    API_CATCH(c)
}
