// Stable counting sort of particles by cell -- sort_particles!
// (grid_sorting.jl:58-113 and :128-182) -- and the gap-closing compaction that
// plays the role of squash_pia! (particles.jl:622-682).
//
// Pipeline (all on the context stream):
//   count   : per live slot, the destination cell (stored key or floor(x/dx));
//             warp-aggregated atomicAdd into counts[cell]
//   scan    : two passes over tiles of cells (launch_scan_cells): exclusive
//             scan of counts -> indexer start1/n_group1, group 2 cleared,
//             cursors zeroed, counts zeroed for reuse
//   scatter : per live slot, position = start1[cell] + ticket (warp-aggregated
//             atomic); idx[position] = slot.  Tickets arrive in any order.
//   gather  : one warp per cell sorts its idx segment ascending (a bitonic
//             network held in registers) -- this restores the reference's
//             stable order exactly -- then moves both 32-byte records of every
//             particle into the other buffer, coalesced on the write side.
// Algorithmic bytes per particle: 64 read + 64 written (+ 16 B of keys/idx).
#include "mz_host.h"
#include "sortnet.cuh"

#include <algorithm>
#include <climits>

using namespace mz;

namespace {

__global__ void k_count(DomainView d, int s, int64_t hw, int mode, double inv_dx)
{
    const SpeciesView& S = d.sp[s];
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < hw; base += stride) {
        int64_t slot = base + lane;
        bool in = slot < hw && S.cell[slot] >= 0;
        unsigned m = __ballot_sync(0xFFFFFFFFu, in);
        if (!in) continue;
        int32_t key;
        if (mode == 1) {
            // get_cell (grid_uniform1D.jl:97-99), 0-based
            double f = floor(S.A.pos[slot].x * inv_dx);
            if (!(f >= 0.0 && f < (double)d.n_cells)) {
                set_status(d, ST_OUTSIDE_GRID);
                f = f < 0.0 || f != f ? 0.0 : (double)(d.n_cells - 1);
            }
            key = (int32_t)f;
            S.key[slot] = key;
        } else {
            key = S.key[slot];
        }
        warp_agg_add(S.counts, key, m);
    }
}

__global__ void k_key_from_cell(DomainView d, int s, int64_t hw)
{
    const SpeciesView& S = d.sp[s];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < hw; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t c = S.cell[i];
        if (c >= 0) S.key[i] = c;
    }
}

// Single-block exclusive scan over n cells.  Writes the indexer (group 1 only)
// and zeroes fill/counts when write_indexer, else writes base_out[c].
// Exclusive scan of per-cell counts in two passes over tiles of SCAN_TILE
// cells (one block of SCAN_THREADS threads per tile, SCAN_PER_THREAD
// consecutive cells per thread): k_scan_tiles sums every tile, k_scan_apply
// adds the sums of the tiles before its own and scans the tile.
constexpr int SCAN_THREADS = 256, SCAN_PER_THREAD = 8, SCAN_TILE = SCAN_THREADS * SCAN_PER_THREAD;
static_assert(SCAN_TILE == MZ_SCAN_TILE, "tile size");

struct ScanArgs {
    int32_t* counts;
    int32_t n;
    Indexer* ind;
    int32_t* fill;
    int32_t* base_out;
    int64_t base_offset;
    int64_t* total_out;
    int write_indexer;
    const Indexer* nlocal_from;  // counts from n1 + n2 of an indexer instead
    int64_t* tile_sums;
    const long long* base_offset_dev;  // added to base_offset when not null (a count the host does not hold)
    const int* abort;                  // nonzero: the fused step was abandoned, write nothing
};

__device__ __forceinline__ int32_t scan_count(const ScanArgs& a, int c)
{
    return a.nlocal_from ? a.nlocal_from[c].n1 + a.nlocal_from[c].n2 : a.counts[c];
}

// block-wide exclusive scan of one value per thread; returns the block total
__device__ __forceinline__ long long block_exclusive_scan(long long v, long long& excl)
{
    __shared__ long long warp_tot[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long u = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += u;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    long long before = 0, total = 0;
#pragma unroll
    for (int k = 0; k < SCAN_THREADS / 32; ++k) {
        const long long t = warp_tot[k];
        before += k < w ? t : 0;
        total += t;
    }
    excl = before + incl - v;
    return total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(ScanArgs a)
{
    if (a.abort && *a.abort) return;
    const int c0 = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
    long long local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; ++k)
        if (c0 + k < a.n) local += scan_count(a, c0 + k);
    long long excl;
    const long long total = block_exclusive_scan(local, excl);
    if (threadIdx.x == 0) a.tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(ScanArgs a)
{
    __shared__ long long prefix_sh;
    if (a.abort && *a.abort) return;
    // sum of the tiles before this one
    long long pre = 0;
    for (int t = threadIdx.x; t < (int)blockIdx.x; t += blockDim.x) pre += a.tile_sums[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pre += __shfl_xor_sync(0xFFFFFFFFu, pre, o);
    if (threadIdx.x == 0) prefix_sh = 0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0 && pre) atomicAdd((unsigned long long*)&prefix_sh, (unsigned long long)pre);
    __syncthreads();
    const long long tile_base = a.base_offset + (a.base_offset_dev ? *a.base_offset_dev : 0ll) + prefix_sh;

    const int c0 = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER_THREAD;
    int32_t cnt[SCAN_PER_THREAD];
    long long local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; ++k) {
        cnt[k] = c0 + k < a.n ? scan_count(a, c0 + k) : 0;
        local += cnt[k];
    }
    long long excl;
    const long long total = block_exclusive_scan(local, excl);
    long long run = tile_base + excl;
#pragma unroll
    for (int k = 0; k < SCAN_PER_THREAD; ++k) {
        const int c = c0 + k;
        if (c >= a.n) break;
        if (a.write_indexer) {
            Indexer p;
            p.start1 = (int32_t)run;
            p.n1 = cnt[k];
            p.start2 = 0;
            p.n2 = 0;
            a.ind[c] = p;
            a.fill[c] = 0;
            a.counts[c] = 0;
        }
        if (a.base_out) a.base_out[c] = (int32_t)run;
        run += cnt[k];
    }
    if (a.total_out && blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *a.total_out = prefix_sh + total;
}

__global__ void k_scatter(DomainView d, int s, int64_t hw)
{
    const SpeciesView& S = d.sp[s];
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < hw; base += stride) {
        int64_t slot = base + lane;
        bool in = slot < hw && S.cell[slot] >= 0;
        unsigned m = __ballot_sync(0xFFFFFFFFu, in);
        if (!in) continue;
        int32_t key = S.key[slot];
        int32_t pos = S.ind[key].start1 + warp_agg_ticket(S.fill, key, m);
        S.idx[pos] = (int32_t)slot;
    }
}

constexpr size_t SORT_GATHER_SMEM = (size_t)8 * SORT_SMEM_KEYS * sizeof(int32_t);  // 64 KB per 256-thread block

__global__ void __launch_bounds__(256) k_sort_gather(DomainView d, int s)
{
    extern __shared__ int32_t sortbuf[];  // SORT_SMEM_KEYS per warp
    const SpeciesView& S = d.sp[s];
    const int warps = (gridDim.x * blockDim.x) >> 5;
    int32_t* mine = sortbuf + (size_t)(threadIdx.x >> 5) * SORT_SMEM_KEYS;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < d.n_cells; c += warps) {
        const Indexer p = S.ind[c];
        sort_gather_segment<false, true>(S, c, p.start1, p.n1, mine);
    }
}

// Compaction: every cell's logical list (group1 then group2) moves to
// [base[c], base[c] + n_local) of the other buffer.
__global__ void __launch_bounds__(256) k_compact_gather(DomainView d, int s, const int32_t* base)
{
    const SpeciesView& S = d.sp[s];
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < d.n_cells; c += warps) {
        const Indexer p = S.ind[c];
        const int32_t nl = p.n1 + p.n2;
        const int32_t b = base[c];
        for (int j = lane; j < nl; j += 32) {
            int64_t dst = (int64_t)b + j;
            copy_particle(S.A, S.B, map_slot(p, j), dst);
            S.cellB[dst] = c;
            S.key[dst] = c;
        }
        __syncwarp();
        if (lane == 0) {
            Indexer q;
            q.start1 = b;
            q.n1 = nl;
            q.start2 = 0;
            q.n2 = 0;
            S.ind[c] = q;
        }
    }
}

__global__ void k_fill_i32(int32_t* p, int64_t n, int32_t v)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = v;
}

}  // namespace

void launch_fill_i32(mz_ctx* c, int32_t* p, int64_t n, int32_t v)
{
    if (n <= 0) return;
    int blocks = (int)std::min<int64_t>(div_up(n, 256), (int64_t)c->num_sms * 8);
    MZ_LAUNCH(c, "fill", k_fill_i32, blocks, 256, 0, p, n, v);
}

void launch_scan_cells(mz_domain* d, int32_t* counts, Indexer* ind, int32_t* fill, int64_t* total_out,
                       bool write_indexer, int32_t* base_out, int64_t base_offset, const Indexer* nlocal_from,
                       const long long* base_offset_dev, const int* abort)
{
    ScanArgs a;
    a.counts = counts;
    a.n = (int32_t)d->n_cells;
    a.ind = ind;
    a.fill = fill;
    a.base_out = base_out;
    a.base_offset = base_offset;
    a.total_out = total_out;
    a.write_indexer = write_indexer ? 1 : 0;
    a.nlocal_from = nlocal_from;
    a.tile_sums = d->d_tile_sums;
    a.base_offset_dev = base_offset_dev;
    a.abort = abort;
    const int tiles = (int)std::max<int64_t>(1, scan_tiles(d->n_cells));
    MZ_LAUNCH(d->ctx, "scan_tiles", k_scan_tiles, tiles, SCAN_THREADS, 0, a);
    MZ_LAUNCH(d->ctx, "scan", k_scan_apply, tiles, SCAN_THREADS, 0, a);
}

static int grid_for(mz_ctx* c, int64_t work, int threads, int per_sm = 8)
{
    return (int)std::max<int64_t>(1, std::min<int64_t>(div_up(work, threads), (int64_t)c->num_sms * per_sm));
}

void launch_sort(mz_domain* d, int s, const mz_grid1d* grid, int64_t* out_index)
{
    mz_ctx* c = d->ctx;
    {
        // the gather's per-warp sort buffers exceed the default shared-memory
        // limit (never called under stream capture: the sort synchronises)
        static bool raised[64] = {false};
        if (c->device < 0 || c->device >= 64 || !raised[c->device]) {
            MZ_CK(cudaFuncSetAttribute(k_sort_gather, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)SORT_GATHER_SMEM));
            if (c->device >= 0 && c->device < 64) raised[c->device] = true;
        }
    }
    SpeciesHost& S = d->sp[s];
    DomainView v = make_view(d);
    const int64_t hw = S.hw;
    std::vector<int32_t> cell_before;
    if (out_index && hw > 0) {
        cell_before.resize(hw);
        MZ_CK(cudaMemcpyAsync(cell_before.data(), S.cell[S.cur], hw * sizeof(int32_t), cudaMemcpyDeviceToHost,
                              c->stream));
    }
    if (hw > 0) {
        int mode = grid ? 1 : 0;
        MZ_LAUNCH(c, "sort_count", k_count, grid_for(c, hw, 256), 256, 0, v, s, hw, mode, grid ? grid->inv_dx : 0.0);
    }
    launch_scan_cells(d, S.counts, S.ind, S.fill, d->d_scalar, true, nullptr, 0, nullptr);
    if (hw > 0) {
        MZ_LAUNCH(c, "sort_scatter", k_scatter, grid_for(c, hw, 256), 256, 0, v, s, hw);
        MZ_LAUNCH(c, "sort_gather", k_sort_gather, grid_for(c, d->n_cells * 32, 256, 16), 256, SORT_GATHER_SMEM, v,
                  s);
    }
    MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    std::vector<int32_t> idx;
    MZ_CK(cudaStreamSynchronize(c->stream));
    int64_t n_total = d->h_scalar[0];
    if (out_index && n_total > 0) {
        idx.resize(n_total);
        MZ_CK(cudaMemcpy(idx.data(), S.idx, n_total * sizeof(int32_t), cudaMemcpyDeviceToHost));
        // logical position of a slot = its rank among live slots
        std::vector<int64_t> rank(hw, -1);
        int64_t r = 0;
        for (int64_t i = 0; i < hw; ++i)
            if (cell_before[i] >= 0) rank[i] = r++;
        // idx segments were sorted in place only in registers; recover the
        // stable order by sorting each cell's segment here as well
        std::vector<mz::Indexer> ind(d->n_cells);
        MZ_CK(cudaMemcpy(ind.data(), S.ind, d->n_cells * sizeof(mz::Indexer), cudaMemcpyDeviceToHost));
        for (int64_t cc = 0; cc < d->n_cells; ++cc)
            std::sort(idx.begin() + ind[cc].start1, idx.begin() + ind[cc].start1 + ind[cc].n1);
        for (int64_t i = 0; i < n_total; ++i) out_index[i] = rank[idx[i]];
    }
    S.n_total = n_total;
    S.hw = n_total;
    S.cur ^= 1;
    S.compact = true;
    S.group2 = false;
}

void launch_compact(mz_domain* d, int s)
{
    mz_ctx* c = d->ctx;
    SpeciesHost& S = d->sp[s];
    if (S.compact) return;
    DomainView v = make_view(d);
    launch_scan_cells(d, S.counts, S.ind, S.fill, d->d_scalar, false, S.work, 0, S.ind);
    MZ_LAUNCH(c, "compact_gather", k_compact_gather, grid_for(c, d->n_cells * 32, 256, 16), 256, 0, v, s, S.work);
    MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    S.n_total = d->h_scalar[0];
    S.hw = S.n_total;
    S.cur ^= 1;
    S.compact = true;
    S.group2 = false;
}

void launch_key_from_cell(mz_domain* d, int s)
{
    mz_ctx* c = d->ctx;
    SpeciesHost& S = d->sp[s];
    if (S.hw <= 0) return;
    DomainView v = make_view(d);
    MZ_LAUNCH(c, "key_from_cell", k_key_from_cell, grid_for(c, S.hw, 256), 256, 0, v, s, S.hw);
}
