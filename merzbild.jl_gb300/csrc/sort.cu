// Stable counting sort of particles by cell -- sort_particles!
// (grid_sorting.jl:58-113 and :128-182) -- and the gap-closing compaction that
// plays the role of squash_pia! (particles.jl:622-682).
//
// Pipeline (all on the context stream):
//   count   : per live slot, the destination cell (stored key or floor(x/dx));
//             warp-aggregated atomicAdd into counts[cell]
//   scan    : one block, exclusive scan of counts -> indexer start1/n_group1,
//             group 2 cleared, cursors zeroed, counts zeroed for reuse
//   scatter : per live slot, position = start1[cell] + ticket (warp-aggregated
//             atomic); idx[position] = slot.  Tickets arrive in any order.
//   gather  : one warp per cell sorts its idx segment ascending (a bitonic
//             network held in registers) -- this restores the reference's
//             stable order exactly -- then moves the 7 FP64 columns of every
//             particle into the other buffer, coalesced on the write side.
// Algorithmic bytes per particle: 56 read + 56 written (+ 16 B of keys/idx).
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
            double f = floor(S.A.x[slot] * inv_dx);
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
__global__ void __launch_bounds__(1024) k_scan(int32_t* counts, int32_t n, Indexer* ind, int32_t* fill,
                                               int32_t* base_out, int64_t base_offset, int64_t* total_out,
                                               int write_indexer, const Indexer* nlocal_from)
{
    __shared__ long long warp_tot[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int chunk = (n + blockDim.x - 1) / blockDim.x;
    const int c0 = min(n, t * chunk), c1 = min(n, c0 + chunk);
    long long local = 0;
    for (int c = c0; c < c1; ++c) local += nlocal_from ? (nlocal_from[c].n1 + nlocal_from[c].n2) : counts[c];
    long long incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        long long v = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    if (w == 0) {
        long long v = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0;
        long long vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            long long u = __shfl_up_sync(0xFFFFFFFFu, vi, o);
            if (lane >= o) vi += u;
        }
        warp_tot[lane] = vi - v;  // exclusive prefix of warp totals
        if (lane == 31 && total_out) *total_out = vi;
    }
    __syncthreads();
    long long run = base_offset + warp_tot[w] + (incl - local);
    for (int c = c0; c < c1; ++c) {
        int32_t cnt = nlocal_from ? (nlocal_from[c].n1 + nlocal_from[c].n2) : counts[c];
        if (write_indexer) {
            Indexer p;
            p.start1 = (int32_t)run;
            p.n1 = cnt;
            p.start2 = 0;
            p.n2 = 0;
            ind[c] = p;
            fill[c] = 0;
            counts[c] = 0;
        }
        if (base_out) base_out[c] = (int32_t)run;
        run += cnt;
    }
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

__global__ void __launch_bounds__(256) k_sort_gather(DomainView d, int s)
{
    const SpeciesView& S = d.sp[s];
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < d.n_cells; c += warps) {
        const Indexer p = S.ind[c];
        sort_gather_segment(S, c, p.start1, p.n1);
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
                       bool write_indexer, int32_t* base_out, int64_t base_offset)
{
    MZ_LAUNCH(d->ctx, "scan", k_scan, 1, 1024, 0, counts, (int32_t)d->n_cells, ind, fill, base_out, base_offset,
              total_out, write_indexer ? 1 : 0, (const Indexer*)nullptr);
}

static int grid_for(mz_ctx* c, int64_t work, int threads, int per_sm = 8)
{
    return (int)std::max<int64_t>(1, std::min<int64_t>(div_up(work, threads), (int64_t)c->num_sms * per_sm));
}

void launch_sort(mz_domain* d, int s, const mz_grid1d* grid, int64_t* out_index)
{
    mz_ctx* c = d->ctx;
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
    MZ_LAUNCH(c, "scan", k_scan, 1, 1024, 0, S.counts, (int32_t)d->n_cells, S.ind, S.fill, (int32_t*)nullptr,
              (int64_t)0, d->d_scalar, 1, (const Indexer*)nullptr);
    if (hw > 0) {
        MZ_LAUNCH(c, "sort_scatter", k_scatter, grid_for(c, hw, 256), 256, 0, v, s, hw);
        MZ_LAUNCH(c, "sort_gather", k_sort_gather, grid_for(c, d->n_cells * 32, 256, 16), 256, 0, v, s);
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
}

void launch_compact(mz_domain* d, int s)
{
    mz_ctx* c = d->ctx;
    SpeciesHost& S = d->sp[s];
    if (S.compact) return;
    DomainView v = make_view(d);
    MZ_LAUNCH(c, "compact_scan", k_scan, 1, 1024, 0, S.counts, (int32_t)d->n_cells, S.ind, S.fill, S.work, (int64_t)0,
              d->d_scalar, 0, (const Indexer*)S.ind);
    MZ_LAUNCH(c, "compact_gather", k_compact_gather, grid_for(c, d->n_cells * 32, 256, 16), 256, 0, v, s, S.work);
    MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
    MZ_CK(cudaStreamSynchronize(c->stream));
    S.n_total = d->h_scalar[0];
    S.hw = S.n_total;
    S.cur ^= 1;
    S.compact = true;
}

void launch_key_from_cell(mz_domain* d, int s)
{
    mz_ctx* c = d->ctx;
    SpeciesHost& S = d->sp[s];
    if (S.hw <= 0) return;
    DomainView v = make_view(d);
    MZ_LAUNCH(c, "key_from_cell", k_key_from_cell, grid_for(c, S.hw, 256), 256, 0, v, s, S.hw);
}
