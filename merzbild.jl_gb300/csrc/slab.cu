// Slab decomposition of a 1-D grid over several GPUs: the particle exchange
// after convection.  The reference moves particles between the cell chunks
// of a multithreaded run with exchange_particles! and
// sort_particles_after_exchange! (parallel.jl:281-532); here one process per
// GPU owns the cells [c0, c0 + n_cells) of the global grid (the domain's
// cells, their streams keyed on the global cell ids through
// mz_set_cell_rng), convects its particles on the global grid and walls, and
// hands the particles that left its slab to the neighbouring ranks.
//
//   mz_slab_extract : stable three-way split of the used slots by global cell
//                     (get_cell, grid_uniform1D.jl:97-99): to the left
//                     neighbour, own, to the right neighbour.  Leaving
//                     particles are staged in slot order and their slots
//                     freed.
//   mz_slab_fetch   : the staged particles to the host, 7 doubles each
//                     (w, vx, vy, vz, x, y, z)
//   mz_slab_insert  : the storage rebuilt as [from the left | own | from the
//                     right], then the stable sort by cell
// so every cell's particles end in the order a single domain over the whole
// grid gives them: the left neighbour's (lower global slots) first, then the
// rank's own, then the right neighbour's.  Streams keyed on global cells and
// this order make a sharded run equal to the single-domain run bit for bit.
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

constexpr int SLAB_THREADS = 256, SLAB_PER = 8, SLAB_TILE = SLAB_THREADS * SLAB_PER;

struct SlabArgs {
    int s;
    int64_t hw;
    double inv_dx;
    int64_t c0, n_global;
    int32_t* tile_counts;  // per tile {left, own, right}, then their exclusive prefixes
    long long* totals;     // {left, own, right}
    double* left;          // staging, 7 doubles per particle
    double* right;
    int32_t* own_rank;     // per slot: rank among the own particles, -1 otherwise
    int32_t* own_cell;     // per slot: local cell of an own particle
};

// 0: to the left neighbour, 1: own (local cell in `local`), 2: to the right
// neighbour, -1: free slot.  Positions map to global cells as get_cell does;
// a particle leaves the global grid only through a wall, so the ends clamp.
__device__ __forceinline__ int classify(const SpeciesView& S, const SlabArgs& a, int n_cells, int64_t slot,
                                        int32_t& local)
{
    if (slot >= a.hw || S.cell[slot] < 0) return -1;
    int64_t g = (int64_t)floor(S.A.pos[slot].x * a.inv_dx);
    g = g < 0 ? 0 : (g >= a.n_global ? a.n_global - 1 : g);
    if (g < a.c0) return 0;
    if (g >= a.c0 + n_cells) return 2;
    local = (int32_t)(g - a.c0);
    return 1;
}

// block-wide exclusive scan of three counters; returns the block totals
__device__ __forceinline__ int3 block_scan3(int3 v, int3& excl)
{
    __shared__ int3 warp_tot[SLAB_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int3 inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xFFFFFFFFu, inc.x, o), y = __shfl_up_sync(0xFFFFFFFFu, inc.y, o),
                  z = __shfl_up_sync(0xFFFFFFFFu, inc.z, o);
        if (lane >= o) {
            inc.x += x;
            inc.y += y;
            inc.z += z;
        }
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    int3 before = make_int3(0, 0, 0), tot = make_int3(0, 0, 0);
#pragma unroll
    for (int k = 0; k < SLAB_THREADS / 32; ++k) {
        const int3 t = warp_tot[k];
        if (k < w) {
            before.x += t.x;
            before.y += t.y;
            before.z += t.z;
        }
        tot.x += t.x;
        tot.y += t.y;
        tot.z += t.z;
    }
    __syncthreads();
    excl = make_int3(before.x + inc.x - v.x, before.y + inc.y - v.y, before.z + inc.z - v.z);
    return tot;
}

// pass 1: per tile of SLAB_TILE consecutive slots, the counts of each class
// (a thread takes SLAB_PER consecutive slots, so tile order is slot order)
__global__ void __launch_bounds__(SLAB_THREADS) k_slab_count(DomainView d, SlabArgs a)
{
    const SpeciesView& S = d.sp[a.s];
    const int64_t tiles = (a.hw + SLAB_TILE - 1) / SLAB_TILE;
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        int3 c = make_int3(0, 0, 0);
        for (int r = 0; r < SLAB_PER; ++r) {
            const int64_t slot = t * SLAB_TILE + (int64_t)threadIdx.x * SLAB_PER + r;
            int32_t local = 0;
            const int k = classify(S, a, d.n_cells, slot, local);
            c.x += k == 0;
            c.y += k == 1;
            c.z += k == 2;
        }
        int3 ex;
        const int3 tot = block_scan3(c, ex);
        if (threadIdx.x == 0) {
            a.tile_counts[3 * t] = tot.x;
            a.tile_counts[3 * t + 1] = tot.y;
            a.tile_counts[3 * t + 2] = tot.z;
        }
    }
}

// pass 2 (one block): exclusive prefixes of the tile counts in place, totals out
__global__ void __launch_bounds__(SLAB_THREADS) k_slab_scan(SlabArgs a, int64_t tiles)
{
    __shared__ long long carry[3];
    if (threadIdx.x < 3) carry[threadIdx.x] = 0;
    __syncthreads();
    for (int64_t t0 = 0; t0 < tiles; t0 += SLAB_THREADS) {
        const int64_t t = t0 + threadIdx.x;
        int3 v = make_int3(0, 0, 0);
        if (t < tiles) v = make_int3(a.tile_counts[3 * t], a.tile_counts[3 * t + 1], a.tile_counts[3 * t + 2]);
        int3 ex;
        const int3 tot = block_scan3(v, ex);
        if (t < tiles) {
            a.tile_counts[3 * t] = (int32_t)(carry[0] + ex.x);
            a.tile_counts[3 * t + 1] = (int32_t)(carry[1] + ex.y);
            a.tile_counts[3 * t + 2] = (int32_t)(carry[2] + ex.z);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            carry[0] += tot.x;
            carry[1] += tot.y;
            carry[2] += tot.z;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        a.totals[0] = carry[0];
        a.totals[1] = carry[1];
        a.totals[2] = carry[2];
    }
}

// pass 3: leaving particles to staging in slot order, their slots freed; own
// particles keep their rank among the own ones and their local cell
__global__ void __launch_bounds__(SLAB_THREADS) k_slab_place(DomainView d, SlabArgs a)
{
    const SpeciesView& S = d.sp[a.s];
    const int64_t tiles = (a.hw + SLAB_TILE - 1) / SLAB_TILE;
    for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
        int kind[SLAB_PER];
        int32_t local[SLAB_PER];
        int3 c = make_int3(0, 0, 0);
#pragma unroll
        for (int r = 0; r < SLAB_PER; ++r) {
            const int64_t slot = t * SLAB_TILE + (int64_t)threadIdx.x * SLAB_PER + r;
            local[r] = 0;
            kind[r] = classify(S, a, d.n_cells, slot, local[r]);
            c.x += kind[r] == 0;
            c.y += kind[r] == 1;
            c.z += kind[r] == 2;
        }
        int3 ex;
        block_scan3(c, ex);
        int3 pos = make_int3(a.tile_counts[3 * t] + ex.x, a.tile_counts[3 * t + 1] + ex.y,
                             a.tile_counts[3 * t + 2] + ex.z);
#pragma unroll
        for (int r = 0; r < SLAB_PER; ++r) {
            const int64_t slot = t * SLAB_TILE + (int64_t)threadIdx.x * SLAB_PER + r;
            if (slot >= a.hw) break;
            if (kind[r] == 1) {
                a.own_rank[slot] = pos.y++;
                a.own_cell[slot] = local[r];
                continue;
            }
            a.own_rank[slot] = -1;
            if (kind[r] < 0) continue;
            double* dst = kind[r] == 0 ? a.left + 7 * (int64_t)pos.x++ : a.right + 7 * (int64_t)pos.z++;
            const PV v = S.A.wv[slot];
            const PX x = S.A.pos[slot];
            dst[0] = v.w;
            dst[1] = v.vx;
            dst[2] = v.vy;
            dst[3] = v.vz;
            dst[4] = x.x;
            dst[5] = x.y;
            dst[6] = x.z;
            S.cell[slot] = -1;
        }
    }
}

// arrivals into buffer B: [0, n_left) from the left, [n_left + n_own, ...)
// from the right, their local cells from their positions
__global__ void k_slab_arrivals(DomainView d, SlabArgs a, const double* in, int64_t n_left, int64_t n_right,
                                int64_t n_own)
{
    const SpeciesView& S = d.sp[a.s];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_left + n_right;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double* src = in + 7 * i;
        const int64_t dst = i < n_left ? i : i + n_own;
        S.B.wv[dst] = PV{src[0], src[1], src[2], src[3]};
        S.B.pos[dst] = PX{src[4], src[5], src[6], 0.0};
        int64_t g = (int64_t)floor(src[4] * a.inv_dx);
        g = g < 0 ? 0 : (g >= a.n_global ? a.n_global - 1 : g);
        int64_t local = g - a.c0;
        if (local < 0 || local >= d.n_cells) {
            // an arrival that crossed a whole neighbour's slab in one step
            set_status(d, ST_OUTSIDE_GRID);
            local = local < 0 ? 0 : d.n_cells - 1;
        }
        S.cellB[dst] = (int32_t)local;
    }
}

// the own particles into buffer B after the arrivals from the left, in slot order
__global__ void k_slab_own(DomainView d, SlabArgs a, int64_t n_left)
{
    const SpeciesView& S = d.sp[a.s];
    for (int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; slot < a.hw;
         slot += (int64_t)gridDim.x * blockDim.x) {
        const int32_t r = a.own_rank[slot];
        if (r < 0) continue;
        const int64_t dst = n_left + r;
        S.B.wv[dst] = S.A.wv[slot];
        S.B.pos[dst] = S.A.pos[slot];
        S.cellB[dst] = a.own_cell[slot];
    }
}

struct SlabState {
    int64_t n_left = -1, n_own = 0, n_right = 0;  // after mz_slab_extract (n_left < 0: none pending)
    bool fetched = false;
};

SlabArgs slab_args(mz_domain* d, int s, const mz_grid1d* g, int64_t c0)
{
    SlabArgs a;
    memset(&a, 0, sizeof a);
    a.s = s;
    a.hw = d->sp[s].hw;
    a.inv_dx = g->inv_dx;
    a.c0 = c0;
    a.n_global = g->n_cells;
    return a;
}

// scratch: per-slot rank and cell, per-tile counts, totals, and the staging
// of leaving / arriving particles (grown on demand)
void ensure(void** p, size_t* have, size_t need)
{
    if (need <= *have) return;
    cudaFree(*p);
    *p = nullptr;
    *have = 0;
    MZ_CK(cudaMalloc(p, need));
    *have = need;
}

}  // namespace

struct mz_slab_scratch {
    void* slots = nullptr;    // 2 int32 per slot
    size_t slots_bytes = 0;
    void* tiles = nullptr;    // 3 int32 per tile + 3 int64 totals
    size_t tiles_bytes = 0;
    void* stage = nullptr;    // 7 doubles per staged particle
    size_t stage_bytes = 0;
    SlabState st[MZ_MAX_SPECIES];
};

void free_slab_scratch(mz_domain* d)
{
    if (!d->slab) return;
    cudaFree(d->slab->slots);
    cudaFree(d->slab->tiles);
    cudaFree(d->slab->stage);
    delete d->slab;
    d->slab = nullptr;
}

extern "C" {

int mz_slab_extract(mz_domain* d, int32_t s, const mz_grid1d* g, int64_t c0, int64_t* n_left, int64_t* n_right)
{
    API_TRY
    MZ_REQUIRE(d && g && n_left && n_right && s >= 0 && s < d->ns, "mz_slab_extract: bad argument");
    MZ_REQUIRE(c0 >= 0 && c0 + d->n_cells <= g->n_cells, "mz_slab_extract: the slab lies outside the global grid");
    MZ_CK(cudaSetDevice(d->ctx->device));
    mz_ctx* c = d->ctx;
    if (!d->slab) d->slab = new mz_slab_scratch();
    mz_slab_scratch& X = *d->slab;
    SpeciesHost& S = d->sp[s];
    SlabArgs a = slab_args(d, s, g, c0);
    const int64_t tiles = std::max<int64_t>(1, div_up(S.hw, SLAB_TILE));
    ensure(&X.slots, &X.slots_bytes, (size_t)std::max<int64_t>(S.hw, 1) * 2 * sizeof(int32_t));
    ensure(&X.tiles, &X.tiles_bytes, (size_t)tiles * 3 * sizeof(int32_t) + 64);
    a.own_rank = static_cast<int32_t*>(X.slots);
    a.own_cell = a.own_rank + std::max<int64_t>(S.hw, 1);
    a.tile_counts = static_cast<int32_t*>(X.tiles);
    a.totals = reinterpret_cast<long long*>(static_cast<char*>(X.tiles) + ((size_t)tiles * 3 * sizeof(int32_t) + 7) / 8 * 8);
    DomainView v = make_view(d);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, (int64_t)c->num_sms * 4));
    MZ_LAUNCH(c, "slab_count", k_slab_count, blocks, SLAB_THREADS, 0, v, a);
    MZ_LAUNCH(c, "slab_scan", k_slab_scan, 1, SLAB_THREADS, 0, a, tiles);
    MZ_CK(cudaMemcpyAsync(d->h_scalar, a.totals, 3 * sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    const int64_t nl = d->h_scalar[0], no = d->h_scalar[1], nr = d->h_scalar[2];
    ensure(&X.stage, &X.stage_bytes, (size_t)std::max<int64_t>(nl + nr, 1) * 7 * sizeof(double));
    a.left = static_cast<double*>(X.stage);
    a.right = a.left + 7 * nl;
    MZ_LAUNCH(c, "slab_place", k_slab_place, blocks, SLAB_THREADS, 0, v, a);
    MZ_CK(cudaStreamSynchronize(c->stream));
    S.n_total = no;
    S.compact = false;
    X.st[s].n_left = nl;
    X.st[s].n_own = no;
    X.st[s].n_right = nr;
    X.st[s].fetched = false;
    *n_left = nl;
    *n_right = nr;
    check_status(d);
    API_CATCH(d->ctx)
}

int mz_slab_fetch(mz_domain* d, int32_t s, double* left, double* right)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns && d->slab && d->slab->st[s].n_left >= 0,
               "mz_slab_fetch: no extraction pending for this species");
    MZ_CK(cudaSetDevice(d->ctx->device));
    const SlabState& st = d->slab->st[s];
    const double* stage = static_cast<const double*>(d->slab->stage);
    MZ_REQUIRE((st.n_left == 0 || left) && (st.n_right == 0 || right), "mz_slab_fetch: NULL output");
    if (st.n_left)
        MZ_CK(cudaMemcpyAsync(left, stage, st.n_left * 7 * sizeof(double), cudaMemcpyDeviceToHost, d->ctx->stream));
    if (st.n_right)
        MZ_CK(cudaMemcpyAsync(right, stage + 7 * st.n_left, st.n_right * 7 * sizeof(double), cudaMemcpyDeviceToHost,
                              d->ctx->stream));
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    d->slab->st[s].fetched = true;
    API_CATCH(d->ctx)
}

int mz_slab_insert(mz_domain* d, int32_t s, const mz_grid1d* g, int64_t c0, const double* from_left, int64_t n_left,
                   const double* from_right, int64_t n_right)
{
    API_TRY
    MZ_REQUIRE(d && g && s >= 0 && s < d->ns && n_left >= 0 && n_right >= 0, "mz_slab_insert: bad argument");
    MZ_REQUIRE((n_left == 0 || from_left) && (n_right == 0 || from_right), "mz_slab_insert: NULL input");
    MZ_REQUIRE(c0 >= 0 && c0 + d->n_cells <= g->n_cells, "mz_slab_insert: the slab lies outside the global grid");
    MZ_REQUIRE(d->slab && d->slab->st[s].n_left >= 0, "mz_slab_insert: no extraction pending for this species");
    MZ_REQUIRE(d->slab->st[s].fetched || d->slab->st[s].n_left + d->slab->st[s].n_right == 0,
               "mz_slab_insert: fetch the leaving particles first (their staging takes the arrivals)");
    MZ_CK(cudaSetDevice(d->ctx->device));
    mz_ctx* c = d->ctx;
    mz_slab_scratch& X = *d->slab;
    SpeciesHost& S = d->sp[s];
    const int64_t no = X.st[s].n_own, total = n_left + no + n_right;
    if (total > S.capacity) reserve_species(d, s, total + total / 8 + 1024);
    ensure(&X.stage, &X.stage_bytes, (size_t)std::max<int64_t>(n_left + n_right, 1) * 7 * sizeof(double));
    double* stage = static_cast<double*>(X.stage);
    if (n_left)
        MZ_CK(cudaMemcpyAsync(stage, from_left, n_left * 7 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (n_right)
        MZ_CK(cudaMemcpyAsync(stage + 7 * n_left, from_right, n_right * 7 * sizeof(double), cudaMemcpyHostToDevice,
                              c->stream));
    SlabArgs a = slab_args(d, s, g, c0);
    a.own_rank = static_cast<int32_t*>(X.slots);
    a.own_cell = a.own_rank + std::max<int64_t>(S.hw, 1);
    DomainView v = make_view(d);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(std::max<int64_t>(S.hw, n_left + n_right), 256),
                                                                  (int64_t)c->num_sms * 8));
    if (n_left + n_right > 0)
        MZ_LAUNCH(c, "slab_arrivals", k_slab_arrivals, blocks, 256, 0, v, a, stage, n_left, n_right, no);
    if (S.hw > 0) MZ_LAUNCH(c, "slab_own", k_slab_own, blocks, 256, 0, v, a, n_left);
    // buffer B now holds [from the left | own | from the right] with cells
    S.cur ^= 1;
    S.hw = S.n_total = total;
    S.compact = false;
    S.group2 = false;
    X.st[s].n_left = -1;
    launch_key_from_cell(d, s);
    launch_sort(d, s, nullptr, nullptr);
    check_status(d);
    API_CATCH(d->ctx)
}

}  // extern "C"
