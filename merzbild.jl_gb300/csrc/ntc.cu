// NTC collisions with VHS cross-sections: ntc! (collision_ntc.jl:338-380,
// :412-453) and ntc_equal_weight! (:479-521, :554-595), including
// collide_2particles_vhs! (:223-270), scatter_vhs! (collision_scattering.jl:17-29)
// and variable-weight splitting.
//
// One group of G lanes (8, 16 or 32; a warp holds 32 / G groups) owns one
// cell.  The reference's candidate loop is sequential: candidates may share
// particles and (sigma g w)_max is raised before each acceptance test.  The
// group evaluates candidates in batches of up to G and keeps the sequential
// semantics exactly:
//   * every candidate j draws from its own Philox stream (i, k, retries,
//     acceptance, scattering angles -- the reference's draw order);
//   * a batch ends before the first candidate that shares a particle with an
//     earlier candidate of the batch, so every candidate sees the velocities
//     the sequential loop would see;
//   * an inclusive warp max-scan of sigma*g*w over the batch reproduces the
//     running maximum each candidate is tested against;
//   * with splitting, a batch ends after the first candidate that splits a
//     particle (the cell grows, so later index draws use the new count).
// Split particles are appended to the cell's group 2 inside a region reserved
// per cell (an exclusive scan of the candidate counts, an upper bound).
#include "cell_ops.cuh"
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

__global__ void k_ntc_prepare(DomainView d, int s1, int s2, uint32_t pc, int cfi, double dt, int cb, int ce,
                              uint32_t step, int split, int32_t* res1, int32_t* res2)
{
    const SpeciesView& S1 = d.sp[s1];
    const SpeciesView& S2 = d.sp[s2];
    // with splitting every cell's reservation is written (the scan reads all);
    // otherwise only the requested range is touched
    const int c_lo = split ? 0 : cb, c_hi = split ? d.n_cells : ce;
    for (int c = c_lo + blockIdx.x * blockDim.x + threadIdx.x; c < c_hi; c += gridDim.x * blockDim.x) {
        int32_t r = 0;
        if (c >= cb && c < ce) {
            const Indexer p1 = S1.ind[c], p2 = S2.ind[c];
            CollisionFactors& cf = d.cf[(size_t)cfi * d.n_cells + c];
            const int32_t nci = ntc_ncoll(d, cf, s1 == s2, p1.n1 + p1.n2, p2.n1 + p2.n2, dt, d.cell_V[c],
                                          cell_seed(d, c), pc, cell_step(d, c, step), cell_rid(d, c));
            r = split ? nci : 0;
        }
        if (res1) res1[c] = r;
        if (res2) res2[c] = r;
    }
}

template <bool EQW, int G>
__global__ void __launch_bounds__(256) k_ntc(DomainView d, int s1, int s2, uint32_t pc, int cfi, int cb, int ce,
                                             uint32_t step, double dw_tol, const int32_t* base1,
                                             const int32_t* base2, const int32_t* res1, const int32_t* res2)
{
    const SpeciesView& S1 = d.sp[s1];
    const SpeciesView& S2 = d.sp[s2];
    const bool single = (s1 == s2);
    const Interaction I = d.inter[s1 + d.n_species * s2];
    const WarpGroup<G> grp;
    const int ngroups = (gridDim.x * blockDim.x) / G;
    for (int c = cb + (int)((blockIdx.x * blockDim.x + threadIdx.x) / G); c < ce; c += ngroups) {
        CollisionFactors* cfp = &d.cf[(size_t)cfi * d.n_cells + c];
        const int32_t ncoll = cfp->n_coll;
        if (ncoll <= 0) continue;
        Indexer p1 = S1.ind[c];
        Indexer p2 = single ? p1 : S2.ind[c];
        const int32_t b1 = EQW ? 0 : base1[c];
        const int32_t b2 = EQW ? 0 : (single ? 0 : base2[c]);
        const NtcResult R =
            (!EQW && single)
                ? ntc_cell_split<G, NTC_SPLIT_VERSIONS>(d, I, c, ncoll, cfp->smax, S1.A, p1, S1.cell, S1.key, b1,
                                                        dw_tol, cell_seed(d, c), pc, cell_step(d, c, step),
                                                        cell_rid(d, c))
                : ntc_cell<EQW, G>(d, I, single, c, ncoll, cfp->smax, S1.A, S2.A, p1, p2, S1.cell, S1.key, S2.cell,
                                   S2.key, b1, b2, dw_tol, cell_seed(d, c), pc, cell_step(d, c, step),
                                   cell_rid(d, c));
        if (!EQW && single) p2 = p1;
        if (grp.rank == 0) {
            cfp->smax = R.smax;
            cfp->n_coll_performed = R.perf;
            cfp->n_eq_w_coll_performed = R.eqw;
            cfp->n_split = R.nsp1 + R.nsp2;
            if (!EQW) {
                S1.ind[c] = p1;
                if (!single) S2.ind[c] = p2;
            }
            atomicAdd(&d.counters->candidates, (unsigned long long)ncoll);
            atomicAdd(&d.counters->accepted, (unsigned long long)R.perf);
            if (!EQW) atomicAdd(&d.counters->splits, (unsigned long long)(R.nsp1 + R.nsp2));
        }
        if (!EQW) {
            // reserved slots not used by splits become dead
            const int32_t r1 = res1[c];
            for (int32_t q = R.nsp1 + grp.rank; q < r1; q += G) S1.cell[b1 + q] = -1;
            if (!single) {
                const int32_t r2 = res2[c];
                for (int32_t q = R.nsp2 + grp.rank; q < r2; q += G) S2.cell[b2 + q] = -1;
            }
        }
    }
}

__global__ void k_split_total(DomainView d, int cfi, int64_t* out)
{
    __shared__ long long sh[32];
    long long t = 0;
    for (int c = threadIdx.x; c < d.n_cells; c += blockDim.x) t += d.cf[(size_t)cfi * d.n_cells + c].n_split;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
        *out = s;
    }
}

}  // namespace

void launch_ntc(mz_domain* d, int s1, int s2, double dt, int64_t cb, int64_t ce, uint64_t step, int32_t flags,
                double dw_tol)
{
    mz_ctx* c = d->ctx;
    const bool eqw = (flags & MZ_NTC_EQUAL_WEIGHT) != 0;
    const uint32_t pc = (uint32_t)(s1 * d->ns + s2);
    const int cfi = s1 + d->ns * s2;
    const bool single = s1 == s2;
    if (!eqw) {
        launch_compact(d, s1);
        if (!single) launch_compact(d, s2);
    }
    SpeciesHost& A = d->sp[s1];
    SpeciesHost& B = d->sp[s2];
    DomainView v = make_view(d);
    const int nc = (int)d->n_cells;
    const int64_t pcells = eqw ? (ce - cb) : nc;
    const int pblocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(pcells, 256), (int64_t)c->num_sms * 8));
    MZ_LAUNCH(c, "ntc_prepare", k_ntc_prepare, pblocks, 256, 0, v, s1, s2, pc, cfi, dt, (int)cb, (int)ce,
              (uint32_t)step, eqw ? 0 : 1, eqw ? (int32_t*)nullptr : A.fill,
              (eqw || single) ? (int32_t*)nullptr : B.fill);
    int64_t tot1 = 0, tot2 = 0;
    if (!eqw) {
        launch_scan_cells(d, A.fill, A.ind, A.fill, d->d_scalar, false, A.work, A.hw);
        if (!single) launch_scan_cells(d, B.fill, B.ind, B.fill, d->d_scalar + 1, false, B.work, B.hw);
        MZ_CK(cudaMemcpyAsync(d->h_scalar, d->d_scalar, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
        MZ_CK(cudaStreamSynchronize(c->stream));
        tot1 = d->h_scalar[0];
        tot2 = single ? 0 : d->h_scalar[1];
        if (A.hw + tot1 > A.capacity) reserve_species(d, s1, A.hw + tot1 + 256);
        if (!single && B.hw + tot2 > B.capacity) reserve_species(d, s2, B.hw + tot2 + 256);
        v = make_view(d);
    }
    const int G = ntc_group_width(ce - cb);
    const int64_t groups_needed = std::max<int64_t>(1, ce - cb);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(groups_needed * G, 256), (int64_t)c->num_sms * 16));
    using KNtc = void (*)(DomainView, int, int, uint32_t, int, int, int, uint32_t, double, const int32_t*,
                          const int32_t*, const int32_t*, const int32_t*);
    const KNtc kern = eqw ? (G == 8 ? k_ntc<true, 8> : G == 16 ? k_ntc<true, 16> : k_ntc<true, 32>)
                          : (G == 8 ? k_ntc<false, 8> : G == 16 ? k_ntc<false, 16> : k_ntc<false, 32>);
    const int32_t* nul = nullptr;
    MZ_LAUNCH(c, "ntc", kern, blocks, 256, 0, v, s1, s2, pc, cfi, (int)cb, (int)ce, (uint32_t)step, dw_tol,
              eqw ? nul : A.work, (eqw || single) ? nul : B.work, eqw ? nul : A.fill,
              (eqw || single) ? nul : B.fill);
    if (!eqw) {
        MZ_LAUNCH(c, "ntc_split_total", k_split_total, 1, 1024, 0, v, cfi, d->d_scalar + 2);
        MZ_CK(cudaMemcpyAsync(d->h_scalar + 2, d->d_scalar + 2, sizeof(int64_t), cudaMemcpyDeviceToHost, c->stream));
        MZ_CK(cudaStreamSynchronize(c->stream));
        // splits land in one species per event; recount per species from the indexers
        A.hw += tot1;
        A.compact = false;
        A.group2 = true;
        if (!single) {
            B.hw += tot2;
            B.compact = false;
            B.group2 = true;
        }
        // exact per-species totals from the indexers
        for (int s : {s1, s2}) {
            std::vector<mz::Indexer> ind(d->n_cells);
            MZ_CK(cudaMemcpy(ind.data(), d->sp[s].ind, d->n_cells * sizeof(mz::Indexer), cudaMemcpyDeviceToHost));
            int64_t n = 0;
            for (auto& p : ind) n += p.n1 + p.n2;
            d->sp[s].n_total = n;
            if (single) break;
        }
    }
}
