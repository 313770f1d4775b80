// Validators of the device indexing -- check_pia_is_correct,
// check_unique_index, check_unique_buffer and count_disordered_particles
// (particles.jl:805-1025) -- for the device layout, and a raw indexer setter
// (a ParticleIndexerArray is mutable data in the reference; its tests build
// inconsistent ones by hand).
//
// Device layout: a cell's group g is the slot range [start_g, start_g + n_g)
// of the species' particle storage; slots [0, hw) are in use, a slot whose
// owner cell is -1 is free (the reference's buffer of free particle indices).
// Every read below stays inside [0, hw): an indexer group that leaves it is
// reported, never followed.
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

// per cell: groups of non-negative size inside [0, hw); the first bad cell
// (1-based) by atomicMin, and the sum of the cells' particle counts
__global__ void k_check_pia(DomainView d, int s, long long hw, unsigned long long* total, int* first_bad)
{
    const SpeciesView& S = d.sp[s];
    long long t = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < d.n_cells; c += gridDim.x * blockDim.x) {
        const Indexer p = S.ind[c];
        bool ok = p.n1 >= 0 && p.n2 >= 0;
        if (ok && p.n1 > 0) ok = p.start1 >= 0 && (long long)p.start1 + p.n1 <= hw;
        if (ok && p.n2 > 0) ok = p.start2 >= 0 && (long long)p.start2 + p.n2 <= hw;
        if (!ok) atomicMin(first_bad, c + 1);
        t += (long long)max(p.n1, 0) + max(p.n2, 0);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
    if ((threadIdx.x & 31) == 0 && t) atomicAdd(total, (unsigned long long)t);
}

// check_unique_index: how many indexer entries point at every slot; a group
// slot outside [0, hw) or on a free slot sets *free_ref
__global__ void k_count_refs(DomainView d, int s, long long hw, int32_t* refs, int* free_ref)
{
    const SpeciesView& S = d.sp[s];
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < d.n_cells; c += warps) {
        const Indexer p = S.ind[c];
        for (int g = 0; g < 2; ++g) {
            const long long st = g == 0 ? p.start1 : p.start2;
            const int n = g == 0 ? p.n1 : p.n2;
            for (int j = lane; j < n; j += 32) {
                const long long slot = st + j;
                if (slot < 0 || slot >= hw) {
                    atomicOr(free_ref, 1);
                    continue;
                }
                atomicAdd(&refs[slot], 1);
                if (S.cell[slot] < 0) atomicOr(free_ref, 1);
            }
        }
    }
}

__global__ void k_max_refs(const int32_t* refs, long long hw, int* max_out)
{
    int m = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < hw; i += (long long)gridDim.x * blockDim.x)
        m = max(m, refs[i]);
    m = __reduce_max_sync(0xFFFFFFFFu, m);
    if ((threadIdx.x & 31) == 0 && m) atomicMax(max_out, m);
}

std::vector<Indexer> download_indexer(mz_domain* d, int s)
{
    std::vector<Indexer> ind(d->n_cells);
    MZ_CK(cudaMemcpyAsync(ind.data(), d->sp[s].ind, d->n_cells * sizeof(Indexer), cudaMemcpyDeviceToHost,
                          d->ctx->stream));
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    return ind;
}

}  // namespace

extern "C" {

int mz_check_indexing(mz_domain* d, int32_t s, int32_t mode, int32_t* ok, int64_t* detail)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns && ok && detail, "mz_check_indexing: bad argument");
    MZ_REQUIRE(mode >= 0 && mode <= 4, "mz_check_indexing: mode must be 0 .. 4");
    MZ_CK(cudaSetDevice(d->ctx->device));
    mz_ctx* c = d->ctx;
    SpeciesHost& S = d->sp[s];
    const long long hw = S.hw;
    DomainView v = make_view(d);
    *ok = 1;
    *detail = 0;
    if (mode == 0) {
        // scratch words: [0] total, [1] first bad cell
        unsigned long long* total = reinterpret_cast<unsigned long long*>(d->d_scalar + 10);
        int* first_bad = reinterpret_cast<int*>(d->d_scalar + 11);
        const int big = 0x7FFFFFFF;
        MZ_CK(cudaMemsetAsync(total, 0, sizeof(unsigned long long), c->stream));
        MZ_CK(cudaMemcpyAsync(first_bad, &big, sizeof(int), cudaMemcpyHostToDevice, c->stream));
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(d->n_cells, 256), (int64_t)c->num_sms * 4));
        MZ_LAUNCH(c, "check_pia", k_check_pia, blocks, 256, 0, v, s, hw, total, first_bad);
        MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar + 10, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
        MZ_CK(cudaStreamSynchronize(c->stream));
        int fb = 0;
        memcpy(&fb, d->h_scalar + 1, sizeof fb);
        if (fb != big) {
            *ok = 0;
            *detail = fb;
        } else if ((int64_t)d->h_scalar[0] != S.n_total) {
            *ok = 0;
            *detail = 0;
        }
    } else if (mode == 1) {
        // per-slot reference counts in the sort's ticket array (rewritten by
        // every sort, unused between calls)
        int* words = reinterpret_cast<int*>(d->d_scalar + 10);  // [0] free slot referenced, [1] max count
        MZ_CK(cudaMemsetAsync(words, 0, 2 * sizeof(int), c->stream));
        if (hw > 0) {
            MZ_CK(cudaMemsetAsync(S.idx, 0, hw * sizeof(int32_t), c->stream));
            const int wblocks =
                (int)std::max<int64_t>(1, std::min<int64_t>(div_up(d->n_cells * 32, 256), (int64_t)c->num_sms * 16));
            MZ_LAUNCH(c, "check_refs", k_count_refs, wblocks, 256, 0, v, s, hw, S.idx, words);
            const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(hw, 256), (int64_t)c->num_sms * 8));
            MZ_LAUNCH(c, "check_refs_max", k_max_refs, blocks, 256, 0, S.idx, hw, words + 1);
        }
        MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar + 10, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
        MZ_CK(cudaStreamSynchronize(c->stream));
        int w[2];
        memcpy(w, d->h_scalar, sizeof w);
        // the reference's return codes: n_index, -n_index (free slots referenced
        // too), -1 (only free slots referenced)
        if (w[1] > 1) {
            *ok = 0;
            *detail = w[0] ? -(int64_t)w[1] : (int64_t)w[1];
        } else if (w[0]) {
            *ok = 0;
            *detail = -1;
        }
    } else if (mode == 2) {
        // check_unique_buffer: free slots are marked per slot (owner -1), so
        // no free slot can be listed twice
    } else {
        // count_disordered_particles: group ranges are contiguous slot
        // ranges, so with per-cell offsets (mode 3) nothing is out of order;
        // without (mode 4) a group is disordered when its first slot differs
        // from its position in the index order (every cell's group 1, then
        // every cell's group 2)
        if (mode == 4) {
            const std::vector<Indexer> ind = download_indexer(d, s);
            int64_t pos = 0, count = 0;
            for (int g = 0; g < 2; ++g)
                for (const Indexer& p : ind) {
                    const int32_t n = g == 0 ? p.n1 : p.n2;
                    const int32_t st = g == 0 ? p.start1 : p.start2;
                    if (n > 0 && st != pos) count += n;
                    pos += std::max(n, 0);
                }
            *detail = count;
        }
    }
    API_CATCH(d->ctx)
}

int mz_set_indexer(mz_domain* d, int32_t s, const mz_particle_indexer* ind, int64_t n_total)
{
    API_TRY
    MZ_REQUIRE(d && s >= 0 && s < d->ns && ind && n_total >= 0, "mz_set_indexer: bad argument");
    MZ_CK(cudaSetDevice(d->ctx->device));
    SpeciesHost& S = d->sp[s];
    std::vector<Indexer> di(d->n_cells);
    int64_t listed = 0;
    for (int64_t c = 0; c < d->n_cells; ++c) {
        const mz_particle_indexer& p = ind[c];
        auto inside = [&](int64_t st, int64_t n) { return n == 0 || (n > 0 && st >= 0 && st + n <= S.hw); };
        MZ_REQUIRE(inside(p.start1, p.n_group1) && inside(p.start2, p.n_group2),
                   "mz_set_indexer: a group lies outside the slots in use");
        // a compaction writes every listed particle once: the storage must hold them
        listed += p.n_group1 + p.n_group2;
        MZ_REQUIRE(listed <= S.capacity, "mz_set_indexer: the groups list more particles than the storage holds");
        di[c] = Indexer{p.n_group1 ? (int32_t)p.start1 : 0, (int32_t)p.n_group1, p.n_group2 ? (int32_t)p.start2 : 0,
                        (int32_t)p.n_group2};
    }
    MZ_CK(cudaMemcpyAsync(S.ind, di.data(), d->n_cells * sizeof(Indexer), cudaMemcpyHostToDevice, d->ctx->stream));
    MZ_CK(cudaStreamSynchronize(d->ctx->stream));
    S.n_total = n_total;
    S.compact = false;
    S.group2 = true;
    API_CATCH(d->ctx)
}

}  // extern "C"
