// Serving loop: continuous batching of independent 0-D solves (the README's
// relaxation problem, README.md:91-106, as a request) on one domain.
//
// Every request owns one cell (a slot) of a server domain for its lifetime.
// Its particles, (sigma g w)_max and random streams live in that slot only:
// the streams are keyed on the request's seed and its own step count (per-cell
// RNG keys with a step offset), and every kernel works per cell, so a
// request's result does not depend on which slot it gets or on what runs
// beside it.  One server step admits queued requests while slots and the
// particle budget allow (compacting storage when dead slots block an
// admission), runs fused 0-D steps (ntc! for every species pair) for all
// running requests at once, and retires requests that reached their step
// count with compute_props! of their last step (the only properties a request
// returns).
//
// Large requests' steps take ~100x longer than small ones' (the candidate
// loop of a cell is a sequential chain of batches whose length grows with
// the cell), so requests run in two lanes by size, each its own domain on its
// own stream: while the large lane runs its steps, the small lane runs batch
// after batch of steps.  A small request then waits for neither the large
// requests' chains nor their admission.
#include "mz_host.h"

#include <algorithm>
#include <cmath>
#include <deque>
#include <unordered_map>

using namespace mz;

namespace {

struct ReqRec {
    mz_request r;
    int32_t state = MZ_REQ_QUEUED;
    int32_t lane = 0;  // 0: small requests, 1: large ones
    int32_t slot = -1;
    int64_t start_step = 0;  // its lane's step count before the request's first step
    mz_request_result res{};
};

// per-slot set-up of admitted requests: RNG keys, volume, (sigma g w)_max
struct AdmitArgs {
    const int32_t* cells;
    int n;
    const uint64_t* seed;
    const uint32_t* offset;
    const double* V;
    const double* smax;  // n x (ns * ns), pair index s1 + ns * s2
};

__global__ void k_admit(DomainView d, AdmitArgs a, uint64_t* cseed, uint32_t* crid, uint32_t* cstep, double* cV)
{
    const int ns = d.n_species;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += gridDim.x * blockDim.x) {
        const int c = a.cells[i];
        cseed[c] = a.seed[i];
        crid[c] = 0;
        cstep[c] = a.offset[i];
        cV[c] = a.V[i];
        for (int p = 0; p < ns * ns; ++p) {
            CollisionFactors& cf = d.cf[(size_t)p * d.n_cells + c];
            cf.smax = a.smax[(size_t)i * ns * ns + p];
            cf.n1 = cf.n2 = cf.n_coll = cf.n_coll_performed = cf.n_eq_w_coll_performed = cf.n_split = 0;
        }
    }
}

// retire: the slot's particles become dead and its lists empty
__global__ void k_release(DomainView d, const int32_t* cells, int n)
{
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += nwarps) {
        const int c = cells[i];
        for (int s = 0; s < d.n_species; ++s) {
            const SpeciesView& S = d.sp[s];
            const Indexer p = S.ind[c];
            for (int j = lane; j < p.n1 + p.n2; j += 32) {
                const int32_t q = map_slot(p, j);
                S.cell[q] = -1;
                S.A.wv[q].w = 0.0;
            }
            __syncwarp();
            if (lane == 0) S.ind[c] = Indexer{0, 0, 0, 0};
        }
    }
}

// compute_props! (physical_props.jl) of the finishing requests only, spread
// over many SMs: one FP64 pipe per SM would take ~0.6 ms for the two passes
// over one 200,000-particle cell.  Each (cell, species) list is cut into fixed
// chunks of LP_CHUNK particles; the chunk sums are combined in chunk order, so
// a request's result depends on its own particles only.
constexpr int LP_CHUNK = 2048;
constexpr int LP_THREADS = 256;

struct ListProps {
    const int32_t* cells;  // cells of the finishing requests
    int n_items;           // cells x species, item = i * n_species + s
    int kmax;              // chunks of the longest list
    double* part;          // [item][chunk][5]: n, sum w vx, sum w vy, sum w vz, sum w |v - u|^2
    double* out;           // [item][6]: np, n, ux, uy, uz, T
};

// block sum of four values in a fixed order (warp butterflies, then warps in order)
__device__ __forceinline__ void lp_block_sum(double (&x)[4], int nv, double* red)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < nv; ++q)
        for (int o = 16; o > 0; o >>= 1) x[q] += __shfl_xor_sync(0xFFFFFFFFu, x[q], o);
    if (lane == 0)
        for (int q = 0; q < nv; ++q) red[4 * wid + q] = x[q];
    __syncthreads();
    for (int q = 0; q < nv; ++q) {
        double t = 0.0;
        for (int w = 0; w < LP_THREADS / 32; ++w) t += red[4 * w + q];
        x[q] = t;
    }
}

__device__ __forceinline__ void lp_mean(const ListProps& a, int item, int nk, double& n, double& ux, double& uy,
                                        double& uz)
{
    const double* pp = a.part + (size_t)item * a.kmax * 5;
    double tx = 0.0, ty = 0.0, tz = 0.0;
    n = 0.0;
    for (int k = 0; k < nk; ++k) {
        n += pp[5 * k];
        tx += pp[5 * k + 1];
        ty += pp[5 * k + 2];
        tz += pp[5 * k + 3];
    }
    ux = uy = uz = 0.0;
    if (n > 0.0) {
        ux = tx / n;
        uy = ty / n;
        uz = tz / n;
    }
}

// pass 1: weight and momentum sums of each chunk
__global__ void __launch_bounds__(LP_THREADS) k_lp_moments(DomainView d, ListProps a)
{
    __shared__ double red[4 * (LP_THREADS / 32)];
    const int item = (int)(blockIdx.x / a.kmax), chunk = (int)(blockIdx.x % a.kmax), ns = d.n_species;
    const SpeciesView& S = d.sp[item % ns];
    const Indexer p = S.ind[a.cells[item / ns]];
    const int32_t tot = p.n1 + p.n2, lo = chunk * LP_CHUNK;
    if (lo >= tot && lo > 0) return;  // block 0 also writes the sums of an empty list
    const int32_t hi = min(tot, lo + LP_CHUNK);
    double x[4] = {0.0, 0.0, 0.0, 0.0};
    for (int32_t j = lo + threadIdx.x; j < hi; j += LP_THREADS) {
        const PV r = S.A.wv[map_slot(p, j)];
        x[0] += r.w;
        x[1] += r.vx * r.w;
        x[2] += r.vy * r.w;
        x[3] += r.vz * r.w;
    }
    lp_block_sum(x, 4, red);
    if (threadIdx.x == 0) {
        double* q = a.part + ((size_t)item * a.kmax + chunk) * 5;
        for (int k = 0; k < 4; ++k) q[k] = x[k];
    }
}

// pass 2: sum w |v - u|^2 of each chunk about the list's mean velocity
__global__ void __launch_bounds__(LP_THREADS) k_lp_energy(DomainView d, ListProps a)
{
    __shared__ double red[4 * (LP_THREADS / 32)];
    const int item = (int)(blockIdx.x / a.kmax), chunk = (int)(blockIdx.x % a.kmax), ns = d.n_species;
    const SpeciesView& S = d.sp[item % ns];
    const Indexer p = S.ind[a.cells[item / ns]];
    const int32_t tot = p.n1 + p.n2, lo = chunk * LP_CHUNK;
    if (lo >= tot && lo > 0) return;  // block 0 also writes the sums of an empty list
    const int32_t hi = min(tot, lo + LP_CHUNK);
    const int nk = min(a.kmax, max(1, (int)((tot + LP_CHUNK - 1) / LP_CHUNK)));
    double n, ux, uy, uz;
    lp_mean(a, item, nk, n, ux, uy, uz);
    double x[4] = {0.0, 0.0, 0.0, 0.0};
    for (int32_t j = lo + threadIdx.x; j < hi; j += LP_THREADS) {
        const PV r = S.A.wv[map_slot(p, j)];
        const double dx = r.vx - ux, dy = r.vy - uy, dz = r.vz - uz;
        x[0] = fma(r.w, (dx * dx + dy * dy) + dz * dz, x[0]);
    }
    lp_block_sum(x, 1, red);
    if (threadIdx.x == 0) a.part[((size_t)item * a.kmax + chunk) * 5 + 4] = x[0];
}

// the list's properties from its chunk sums, one thread per list
__global__ void k_lp_finish(DomainView d, ListProps a)
{
    const int item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= a.n_items) return;
    const int ns = d.n_species;
    const SpeciesView& S = d.sp[item % ns];
    const Indexer p = S.ind[a.cells[item / ns]];
    const int32_t tot = p.n1 + p.n2;
    const int nk = min(a.kmax, max(1, (int)((tot + LP_CHUNK - 1) / LP_CHUNK)));
    double n, ux, uy, uz;
    lp_mean(a, item, nk, n, ux, uy, uz);
    double E = 0.0;
    for (int k = 0; k < nk; ++k) E += a.part[((size_t)item * a.kmax + k) * 5 + 4];
    double* o = a.out + (size_t)item * 6;
    o[0] = (double)tot;
    o[1] = n;
    o[2] = ux;
    o[3] = uy;
    o[4] = uz;
    o[5] = n > 0.0 ? (2.0 / 3.0) * (E * (0.5 * S.mass / (n * K_B))) : 0.0;
}

// estimate_sigma_g_w_max (collision_utils.jl:418-423)
double sigma_g_w_max_estimate(const Interaction& I, double m1, double m2, double T1, double T2, double Fnum)
{
    const double g = 0.5 * (std::sqrt(2.0 * T1 * K_B / m1) + std::sqrt(2.0 * T2 * K_B / m2));
    const double sigma = I.vhs_factor * std::pow(g, std::fma(-2.0, I.vhs_o, 1.0));
    return sigma * g * Fnum;
}

}  // namespace

// One lane: a domain of max_requests cells on its own stream, with its own
// admission queue, slots and step count.
struct ServerLane {
    mz_ctx* ctx = nullptr;     // the lane's own context (streams, events)
    bool own_ctx = false;
    mz_domain* dom = nullptr;
    int64_t step = 0;          // steps this lane has run
    std::deque<int64_t> queue;
    std::vector<int64_t> slot_req;  // request id per slot, 0 = free
    std::vector<int64_t> free_slots;
    std::vector<int64_t> running;   // ids of admitted, unfinished requests
    cudaEvent_t done = nullptr;     // end of the lane's last launched steps
    // device scratch for admissions / retirements
    int32_t* d_cells = nullptr;
    double* d_part = nullptr;  // chunk sums of the finishing requests' props
    int64_t part_cap = 0;      // doubles in d_part
    double* d_lp = nullptr;    // their properties, 6 per (request, species)
    uint64_t* d_seed = nullptr;
    uint32_t* d_off = nullptr;
    double* d_V = nullptr;
    double* d_smax = nullptr;
};

struct mz_server_s {
    mz_ctx* ctx = nullptr;
    int32_t ns = 0;
    int64_t slots = 0;
    double dt = 0.0;
    int64_t next_id = 1;
    // requests of at least `split` particles (all species) run in lane 1,
    // smaller ones in lane 0, each lane stepping at its own pace; 0: lane 0 only
    int64_t split = 4096;
    ServerLane lane[2];
    std::unordered_map<int64_t, ReqRec> reqs;
    std::vector<int64_t> retired;   // ids retired by the last mz_server_step(_many) call
    int64_t particle_steps = 0;
    // admission by free device memory (created with capacity 0): the lanes'
    // particle storage grows at admission while cudaMemGetInfo's free bytes,
    // less `headroom`, cover the larger storage; otherwise the request waits
    bool hbm = false;
    int64_t headroom = (int64_t)2 << 30;
};

namespace {

void ensure_rng_arrays(mz_domain* d)
{
    const int64_t n = d->n_cells;
    if (!d->d_cell_seed) {
        MZ_CK(cudaMalloc(&d->d_cell_seed, n * sizeof(uint64_t)));
        MZ_CK(cudaMemsetAsync(d->d_cell_seed, 0, n * sizeof(uint64_t), d->ctx->stream));
    }
    if (!d->d_cell_rid) {
        MZ_CK(cudaMalloc(&d->d_cell_rid, n * sizeof(uint32_t)));
        MZ_CK(cudaMemsetAsync(d->d_cell_rid, 0, n * sizeof(uint32_t), d->ctx->stream));
    }
    if (!d->d_cell_step) {
        MZ_CK(cudaMalloc(&d->d_cell_step, n * sizeof(uint32_t)));
        MZ_CK(cudaMemsetAsync(d->d_cell_step, 0, n * sizeof(uint32_t), d->ctx->stream));
    }
}

// device bytes one particle slot of a species holds: two buffers of both
// 32-byte records and the owner cell, plus the sort key and ticket
constexpr int64_t SLOT_BYTES = 2 * (int64_t)(sizeof(PV) + sizeof(PX) + sizeof(int32_t)) + 2 * (int64_t)sizeof(int32_t);

// free-memory admission: grow species s of lane domain d to hold `need`
// slots if the device's free memory less the headroom allows (the old
// storage is freed after the copy, so the new one must fit beside it)
bool grow_for(mz_server* sv, mz_domain* d, int s, int64_t need)
{
    if (!sv->hbm) return false;
    size_t free_b = 0, total_b = 0;
    MZ_CK(cudaMemGetInfo(&free_b, &total_b));
    const int64_t avail = (int64_t)free_b - sv->headroom;
    const int64_t cap = d->sp[s].capacity;
    for (const int64_t want : {std::max<int64_t>(need, 2 * cap) + 1024, need + 1024}) {
        if (want * SLOT_BYTES <= avail && want < (1ll << 31) - 2048) {
            reserve_species(d, s, want);
            return true;
        }
    }
    return false;
}

// admit queued requests while slots and storage allow; FIFO, no overtaking
void admit(mz_server* sv, ServerLane& L)
{
    mz_domain* d = L.dom;
    const int ns = sv->ns;
    std::vector<int32_t> cells;
    std::vector<uint64_t> seeds;
    std::vector<uint32_t> offs;
    std::vector<double> Vs, smax;
    std::vector<std::vector<int64_t>> counts(ns, std::vector<int64_t>(d->n_cells, 0));
    std::vector<double> T3(3 * d->n_cells * ns, 0.0), F(d->n_cells * ns, 0.0);
    int64_t need[MZ_MAX_SPECIES] = {0, 0, 0, 0};
    while (!L.queue.empty() && !L.free_slots.empty()) {
        const int64_t id = L.queue.front();
        ReqRec& q = sv->reqs.at(id);
        bool fits = true;
        for (int s = 0; s < ns && fits; ++s) {
            SpeciesHost& S = d->sp[s];
            const int64_t want = need[s] + q.r.count[s];
            if (S.hw + want > S.capacity) {
                // dead slots of retired requests block the admission: compact
                if (S.n_total + want <= S.capacity && need[s] == 0 && !S.compact) launch_compact(d, s);
                // grow the storage into free device memory, or wait
                if (S.hw + want > S.capacity && !grow_for(sv, d, s, S.hw + want)) fits = false;
            }
        }
        if (!fits) break;
        L.queue.pop_front();
        const int32_t slot = (int32_t)L.free_slots.back();
        L.free_slots.pop_back();
        q.state = MZ_REQ_RUNNING;
        q.slot = slot;
        q.start_step = L.step;
        L.slot_req[slot] = id;
        L.running.push_back(id);
        cells.push_back(slot);
        seeds.push_back(q.r.seed);
        offs.push_back((uint32_t)L.step);
        Vs.push_back(q.r.V);
        for (int s2 = 0; s2 < ns; ++s2)
            for (int s1 = 0; s1 < ns; ++s1) {
                const double T1 = q.r.T[s1] > 0 ? q.r.T[s1] : 300.0, T2 = q.r.T[s2] > 0 ? q.r.T[s2] : 300.0;
                smax.push_back(sigma_g_w_max_estimate(d->inter[s1 + ns * s2], d->mass[s1], d->mass[s2], T1, T2,
                                                      q.r.Fnum));
            }
        for (int s = 0; s < ns; ++s) {
            counts[s][slot] = q.r.count[s];
            need[s] += q.r.count[s];
            for (int k = 0; k < 3; ++k) T3[(size_t)s * 3 * d->n_cells + 3 * slot + k] = q.r.T[s];
            F[(size_t)s * d->n_cells + slot] = q.r.Fnum;
        }
    }
    if (cells.empty()) return;
    const int n = (int)cells.size();
    mz_ctx* c = L.ctx;
    MZ_CK(cudaMemcpyAsync(L.d_cells, cells.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(L.d_seed, seeds.data(), n * sizeof(uint64_t), cudaMemcpyHostToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(L.d_off, offs.data(), n * sizeof(uint32_t), cudaMemcpyHostToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(L.d_V, Vs.data(), n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    MZ_CK(cudaMemcpyAsync(L.d_smax, smax.data(), smax.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    AdmitArgs a{L.d_cells, n, L.d_seed, L.d_off, L.d_V, L.d_smax};
    DomainView v = make_view(d);
    MZ_LAUNCH(c, "server_admit", k_admit, (int)div_up(n, 128), 128, 0, v, a, d->d_cell_seed, d->d_cell_rid,
              d->d_cell_step, d->d_V);
    // initial particles of the admitted requests (streams of step 0 of each)
    for (int s = 0; s < ns; ++s) {
        if (need[s] == 0) continue;
        launch_sample_cells(d, s, counts[s].data(), nullptr, T3.data() + (size_t)s * 3 * d->n_cells, nullptr,
                            F.data() + (size_t)s * d->n_cells, 0.0, nullptr, 0, (uint64_t)L.step);
        d->sp[s].compact = false;
    }
}

// Launch the lane's next steps on its stream without waiting: as many as
// every running request still needs, at most max_steps (no request steps
// past its end).  Returns the number of steps (0: nothing runs).
int64_t launch_lane(mz_server* sv, ServerLane& L, int64_t max_steps)
{
    if (L.running.empty()) return 0;
    mz_step_plan plan;
    memset(&plan, 0, sizeof plan);
    plan.dims = 0;
    plan.collide = 1;
    plan.equal_weight = 1;
    plan.props = 0;  // compute_props! of the finishing requests runs after the steps
    plan.dt = sv->dt;
    plan.dw_tol = 1e-16;
    plan.step0 = (uint64_t)L.step;
    plan.use_graph = 0;
    int64_t k = max_steps;
    for (int64_t id : L.running) {
        const ReqRec& q = sv->reqs.at(id);
        k = std::min<int64_t>(k, q.r.n_steps - (L.step - q.start_step));
    }
    k = std::max<int64_t>(k, 1);
    launch_step(L.dom, &plan, k, nullptr, nullptr);
    MZ_CK(cudaEventRecord(L.done, L.ctx->stream));
    return k;
}

// Book the lane's k launched steps and retire the requests they finished:
// compute_props! of their last step over their cells only, then release.
// Returns the number retired.
int64_t finish_lane(mz_server* sv, ServerLane& L, int64_t k)
{
    if (k <= 0) return 0;
    mz_domain* d = L.dom;
    mz_ctx* c = L.ctx;
    const int ns = sv->ns;
    L.step += k;
    std::vector<int64_t> done;
    for (int64_t id : L.running) {
        ReqRec& q = sv->reqs.at(id);
        q.res.steps_done = L.step - q.start_step;
        for (int s = 0; s < ns; ++s) sv->particle_steps += q.r.count[s] * k;
        if (q.res.steps_done >= q.r.n_steps) done.push_back(id);
    }
    if (done.empty()) return 0;
    std::vector<int32_t> cells;
    int64_t kmax = 1;
    for (int64_t id : done) {
        const ReqRec& q = sv->reqs.at(id);
        cells.push_back((int32_t)q.slot);
        for (int s = 0; s < ns; ++s) kmax = std::max<int64_t>(kmax, div_up(q.r.count[s], LP_CHUNK));
    }
    const int n_items = (int)cells.size() * ns;
    MZ_REQUIRE((int64_t)n_items * kmax < INT32_MAX, "mz_server_step: too many particles finishing at once");
    if ((int64_t)n_items * kmax * 5 > L.part_cap) {
        cudaFree(L.d_part);
        L.d_part = nullptr;
        L.part_cap = 0;
        const int64_t cap = std::max<int64_t>((int64_t)n_items * kmax * 5, 1 << 16);
        MZ_CK(cudaMalloc(&L.d_part, cap * sizeof(double)));
        L.part_cap = cap;
    }
    MZ_CK(cudaMemcpyAsync(L.d_cells, cells.data(), cells.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                          c->stream));
    ListProps lp{L.d_cells, n_items, (int)kmax, L.d_part, L.d_lp};
    DomainView vp = make_view(d);
    const int lg = (int)(n_items * kmax);  // one block per (request, species, chunk)
    MZ_LAUNCH(c, "server_props_moments", k_lp_moments, lg, LP_THREADS, 0, vp, lp);
    MZ_LAUNCH(c, "server_props_energy", k_lp_energy, lg, LP_THREADS, 0, vp, lp);
    MZ_LAUNCH(c, "server_props_finish", k_lp_finish, (int)div_up(n_items, 128), 128, 0, vp, lp);
    std::vector<double> o((size_t)n_items * 6);
    MZ_CK(cudaMemcpyAsync(o.data(), L.d_lp, o.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    int i = 0;
    for (int64_t id : done) {
        ReqRec& q = sv->reqs.at(id);
        const int64_t slot = q.slot;
        for (int s = 0; s < ns; ++s) {
            const double* r = o.data() + ((size_t)i * ns + s) * 6;
            q.res.np[s] = (int64_t)r[0];
            q.res.n[s] = r[1];
            for (int a = 0; a < 3; ++a) q.res.v[s][a] = r[2 + a];
            q.res.T[s] = r[5];
        }
        ++i;
        q.res.steps_done = q.r.n_steps;
        q.state = MZ_REQ_DONE;
        sv->retired.push_back(id);
        L.slot_req[slot] = 0;
        L.free_slots.push_back(slot);
        for (int s = 0; s < ns; ++s) d->sp[s].n_total -= q.r.count[s];
    }
    DomainView vv = make_view(d);
    MZ_LAUNCH(c, "server_release", k_release, (int)div_up((int64_t)cells.size() * 32, 256), 256, 0, vv, L.d_cells,
              (int)cells.size());
    for (int s = 0; s < ns; ++s) d->sp[s].compact = false;
    L.running.erase(std::remove_if(L.running.begin(), L.running.end(),
                                   [&](int64_t id) { return sv->reqs.at(id).state == MZ_REQ_DONE; }),
                    L.running.end());
    return (int64_t)done.size();
}

void lane_init(mz_server* sv, ServerLane& L, mz_ctx* c, bool own, int64_t max_requests, const int64_t* capacity,
               const double* mass, const mz_interaction* inter)
{
    L.ctx = c;
    L.own_ctx = own;
    int rc = mz_domain_create(c, max_requests, sv->ns, capacity, &L.dom);
    if (rc == MZ_OK) rc = mz_set_species(L.dom, mass);
    if (rc == MZ_OK) rc = mz_set_interactions(L.dom, inter);
    if (rc != MZ_OK) throw MzError(rc, "mz_server_create: " + c->last_error);
    ensure_rng_arrays(L.dom);
    L.slot_req.assign(max_requests, 0);
    for (int64_t s = max_requests - 1; s >= 0; --s) L.free_slots.push_back(s);
    MZ_CK(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming));
    MZ_CK(cudaMalloc(&L.d_cells, max_requests * sizeof(int32_t)));
    MZ_CK(cudaMalloc(&L.d_lp, max_requests * sv->ns * 6 * sizeof(double)));
    MZ_CK(cudaMalloc(&L.d_seed, max_requests * sizeof(uint64_t)));
    MZ_CK(cudaMalloc(&L.d_off, max_requests * sizeof(uint32_t)));
    MZ_CK(cudaMalloc(&L.d_V, max_requests * sizeof(double)));
    MZ_CK(cudaMalloc(&L.d_smax, max_requests * sv->ns * sv->ns * sizeof(double)));
}

void lane_free(ServerLane& L)
{
    if (!L.ctx) return;
    cudaStreamSynchronize(L.ctx->stream);
    cudaFree(L.d_cells);
    cudaFree(L.d_part);
    cudaFree(L.d_lp);
    cudaFree(L.d_seed);
    cudaFree(L.d_off);
    cudaFree(L.d_V);
    cudaFree(L.d_smax);
    if (L.done) cudaEventDestroy(L.done);
    if (L.dom) mz_domain_destroy(L.dom);
    if (L.own_ctx) mz_ctx_destroy(L.ctx);
    L = ServerLane();
}

}  // namespace

extern "C" {

int mz_server_create(mz_ctx* c, int32_t n_species, const double* mass, const mz_interaction* inter, double dt,
                     int64_t max_requests, const int64_t* capacity, mz_server** out)
{
    API_TRY
    MZ_REQUIRE(c && out && mass && inter && capacity, "mz_server_create: NULL argument");
    MZ_REQUIRE(n_species >= 1 && n_species <= MZ_MAX_SPECIES, "mz_server_create: bad species count");
    MZ_REQUIRE(max_requests >= 1 && max_requests < (1 << 24), "mz_server_create: bad max_requests");
    MZ_REQUIRE(dt > 0.0, "mz_server_create: dt must be positive");
    struct Guard {  // frees a partly built server when set-up throws
        mz_server* p = nullptr;
        ~Guard()
        {
            if (!p) return;
            lane_free(p->lane[0]);
            lane_free(p->lane[1]);
            delete p;
        }
    } guard;
    mz_server* sv = guard.p = new mz_server_s();
    sv->ctx = c;
    sv->ns = n_species;
    sv->slots = max_requests;
    sv->dt = dt;
    int64_t cap[MZ_MAX_SPECIES];
    for (int s = 0; s < n_species; ++s) {
        // capacity 0: admission by free device memory, storage grown on demand
        if (capacity[s] <= 0) sv->hbm = true;
        cap[s] = capacity[s] > 0 ? capacity[s] : 4096;
    }
    // each lane on streams of its own, so that the two overlap
    for (int l = 0; l < 2; ++l) {
        mz_ctx* cl = nullptr;
        const int rc = mz_ctx_create(c->device, &cl);
        if (rc != MZ_OK) throw MzError(rc, "mz_server_create: lane streams");
        sv->lane[l].ctx = cl;  // freed with the lane if the set-up throws
        sv->lane[l].own_ctx = true;
        lane_init(sv, sv->lane[l], cl, true, max_requests, cap, mass, inter);
    }
    *out = sv;
    guard.p = nullptr;
    API_CATCH(c)
}

int mz_server_destroy(mz_server* sv)
{
    if (!sv) return MZ_OK;
    cudaSetDevice(sv->ctx->device);
    lane_free(sv->lane[0]);
    lane_free(sv->lane[1]);
    delete sv;
    return MZ_OK;
}

int mz_server_set_hbm_headroom(mz_server* sv, int64_t bytes)
{
    API_TRY
    MZ_REQUIRE(sv && bytes >= 0, "mz_server_set_hbm_headroom: bad argument");
    sv->headroom = bytes;
    API_CATCH(sv ? sv->ctx : nullptr)
}

/* requests of at least `particles` particles (all species) run in the lane
 * of large requests; 0 puts every request in one lane */
int mz_server_set_lane_split(mz_server* sv, int64_t particles)
{
    API_TRY
    MZ_REQUIRE(sv && particles >= 0, "mz_server_set_lane_split: bad argument");
    sv->split = particles;
    API_CATCH(sv ? sv->ctx : nullptr)
}

int mz_server_submit(mz_server* sv, const mz_request* r, int64_t* id)
{
    API_TRY
    MZ_REQUIRE(sv && r && id, "mz_server_submit: NULL argument");
    MZ_REQUIRE(r->n_steps >= 1 && r->Fnum > 0.0 && r->V > 0.0, "mz_server_submit: bad request");
    size_t free_b = 0, total_b = 0;
    if (sv->hbm) MZ_CK(cudaMemGetInfo(&free_b, &total_b));
    for (int s = 0; s < sv->ns; ++s) {
        if (sv->hbm)
            MZ_REQUIRE(r->count[s] >= 0 && r->count[s] < (1ll << 31) - 4096 &&
                           r->count[s] * SLOT_BYTES <= (int64_t)total_b - sv->headroom,
                       "mz_server_submit: request larger than the device memory less the headroom");
        else
            MZ_REQUIRE(r->count[s] >= 0 && r->count[s] <= sv->lane[0].dom->sp[s].capacity,
                       "mz_server_submit: request larger than the particle budget");
        MZ_REQUIRE(r->count[s] == 0 || r->T[s] > 0.0, "mz_server_submit: temperature must be positive");
    }
    int64_t total = 0;
    for (int s = 0; s < sv->ns; ++s) total += r->count[s];
    ReqRec q;
    q.r = *r;
    q.lane = sv->split > 0 && total >= sv->split ? 1 : 0;
    q.res.id = sv->next_id;
    const int64_t k = sv->next_id++;
    sv->reqs.emplace(k, q);
    sv->lane[q.lane].queue.push_back(k);
    *id = k;
    API_CATCH(sv->ctx)
}

int mz_server_step_many(mz_server* sv, int64_t max_steps, int64_t* n_steps, int64_t* n_running, int64_t* n_queued,
                        int64_t* n_retired)
{
    API_TRY
    MZ_REQUIRE(sv && max_steps >= 1, "mz_server_step_many: bad argument");
    if (n_steps) *n_steps = 0;
    MZ_CK(cudaSetDevice(sv->ctx->device));
    sv->retired.clear();
    ServerLane& small = sv->lane[0];
    ServerLane& large = sv->lane[1];
    // the large requests' steps run on their stream; meanwhile the small
    // requests' lane steps again and again (retiring and admitting between
    // its launches) until the large lane is done, so small requests do not
    // wait for the long collision chains of large cells
    admit(sv, large);
    const int64_t kl = launch_lane(sv, large, max_steps);
    int64_t ks = 0;
    for (;;) {
        admit(sv, small);
        const int64_t k = launch_lane(sv, small, max_steps);
        if (k > 0) {
            MZ_CK(cudaEventSynchronize(small.done));
            finish_lane(sv, small, k);
            ks += k;
        }
        if (kl == 0 || k == 0) break;
        const cudaError_t q = cudaEventQuery(large.done);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) MZ_CK(q);
        if (cudaPeekAtLastError() == cudaErrorNotReady) (void)cudaGetLastError();  // not a failure
    }
    if (kl > 0) {
        MZ_CK(cudaEventSynchronize(large.done));
        finish_lane(sv, large, kl);
    }
    if (n_steps) *n_steps = std::max(kl, ks);
    if (n_running) *n_running = (int64_t)(small.running.size() + large.running.size());
    if (n_queued) *n_queued = (int64_t)(small.queue.size() + large.queue.size());
    if (n_retired) *n_retired = (int64_t)sv->retired.size();
    check_status(small.dom);
    check_status(large.dom);
    API_CATCH(sv->ctx)
}

int mz_server_step(mz_server* sv, int64_t* n_running, int64_t* n_queued, int64_t* n_retired)
{
    return mz_server_step_many(sv, 1, nullptr, n_running, n_queued, n_retired);
}

int mz_server_result(mz_server* sv, int64_t id, mz_request_result* out)
{
    API_TRY
    MZ_REQUIRE(sv && out, "mz_server_result: NULL argument");
    auto it = sv->reqs.find(id);
    MZ_REQUIRE(it != sv->reqs.end(), "mz_server_result: unknown request");
    *out = it->second.res;
    out->id = id;
    out->state = it->second.state;
    if (it->second.state == MZ_REQ_RUNNING)
        out->steps_done = sv->lane[it->second.lane].step - it->second.start_step;
    API_CATCH(sv->ctx)
}

int mz_server_retired(mz_server* sv, int64_t max_ids, int64_t* ids, int64_t* n)
{
    API_TRY
    MZ_REQUIRE(sv && n && (max_ids == 0 || ids), "mz_server_retired: NULL argument");
    *n = (int64_t)sv->retired.size();
    for (int64_t i = 0; i < std::min<int64_t>(max_ids, *n); ++i) ids[i] = sv->retired[i];
    API_CATCH(sv->ctx)
}

int mz_server_info(mz_server* sv, int64_t* steps_run, int64_t* particle_steps)
{
    API_TRY
    MZ_REQUIRE(sv, "mz_server_info: NULL server");
    if (steps_run) *steps_run = std::max(sv->lane[0].step, sv->lane[1].step);
    if (particle_steps) *particle_steps = sv->particle_steps;
    API_CATCH(sv->ctx)
}

}  // extern "C"
