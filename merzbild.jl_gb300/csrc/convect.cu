// 1-D convection with Maxwell walls: convect_single_particle!
// (convection_1D.jl:17-54), convect_particles! (:130-157),
// convect_particles_and_compute_cell! (:225-255), reflect_particle_x! /
// diffuse_reflection_x! / specular_reflection_x! (boundary_conditions.jl:63-121).
//
// One thread per slot.  A particle's random stream is keyed on (cell, position
// j in the cell's logical list), so the result does not depend on the
// physical layout.  Algorithmic bytes per particle: read x, vx (16) + write x
// (8); wall hitters also read/write vy, vz.
#include "cell_ops.cuh"
#include "mz_host.h"

#include <algorithm>

using namespace mz;

namespace {

__global__ void __launch_bounds__(256) k_convect(DomainView d, int s, int64_t hw, WallView W, double dt, uint32_t step,
                                                 int compute_cell, double* surf)
{
    const SpeciesView& S = d.sp[s];
    unsigned long long my_hits = 0;
    bool cap = false;
    SurfAcc acc = {};
    for (int64_t slot = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; slot < hw;
         slot += (int64_t)gridDim.x * blockDim.x) {
        const int32_t c = S.cell[slot];
        if (c < 0) continue;
        const Indexer p = S.ind[c];
        const int32_t j = (slot >= p.start1 && slot < (int64_t)p.start1 + p.n1) ? (int32_t)(slot - p.start1)
                                                                                  : p.n1 + (int32_t)(slot - p.start2);
        Stream st;
        st.init(cell_seed(d, c), TAG_CONVECT, (uint32_t)s, cell_step(d, c, step), cell_rid(d, c), (uint32_t)j);
        double x = S.A.pos[slot].x;
        double vx = S.A.wv[slot].vx;
        const double xn = fma(vx, dt, x);
        if (!move_free(W, xn, x)) {
            const PV r = S.A.wv[slot];
            double vy = r.vy, vz = r.vz;
            my_hits += convect_walls(st, W, s, x, vx, vy, vz, dt, cap, surf ? &acc : nullptr, r.w);
            S.A.wv[slot] = PV{r.w, vx, vy, vz};
        }
        S.A.pos[slot].x = x;
        if (compute_cell) S.key[slot] = cell_of(d, x, W.inv_dx);
    }
    if (cap) set_status(d, ST_WALL_HITS);
    if (my_hits) atomicAdd(&d.counters->wall_hits, my_hits);
    if (surf) surf_flush(acc, surf, my_hits != 0);
}

// The same per-particle work for the fused variable-weight step: slots
// [0, *hw_dev) (the count is on the device), dead slots skipped, the RNG step
// read from device memory, and the destination cell of every particle both
// stored (key) and counted for the next sort (warp-aggregated atomics).
__global__ void __launch_bounds__(256) k_convect_count(DomainView d, int s, const long long* hw_dev, WallView W,
                                                       double dt, const uint32_t* step_ptr, const int* abort,
                                                       double* surf)
{
    if (*abort) return;
    const SpeciesView& S = d.sp[s];
    const int64_t hw = *hw_dev;
    const uint32_t step = *step_ptr;
    unsigned long long my_hits = 0;
    bool cap = false;
    SurfAcc acc = {};
    const int lane = threadIdx.x & 31;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < hw; base += stride) {
        const int64_t slot = base + lane;
        const int32_t c = slot < hw ? S.cell[slot] : -1;
        const bool live = c >= 0;
        int32_t key = 0;
        if (live) {
            const Indexer p = S.ind[c];
            const int32_t j = (slot >= p.start1 && slot < (int64_t)p.start1 + p.n1) ? (int32_t)(slot - p.start1)
                                                                                      : p.n1 + (int32_t)(slot - p.start2);
            double x = S.A.pos[slot].x;
            double vx = S.A.wv[slot].vx;
            const double xn = fma(vx, dt, x);
            if (!move_free(W, xn, x)) {
                Stream st;
                st.init(cell_seed(d, c), TAG_CONVECT, (uint32_t)s, cell_step(d, c, step), cell_rid(d, c),
                        (uint32_t)j);
                const PV r = S.A.wv[slot];
                double vy = r.vy, vz = r.vz;
                my_hits += convect_walls(st, W, s, x, vx, vy, vz, dt, cap, surf ? &acc : nullptr, r.w);
                S.A.wv[slot] = PV{r.w, vx, vy, vz};
            }
            S.A.pos[slot].x = x;
            key = cell_of(d, x, W.inv_dx);
            S.key[slot] = key;
        }
        const unsigned m = __ballot_sync(0xFFFFFFFFu, live);
        if (live) warp_agg_add(S.counts, key, m);
    }
    if (cap) set_status(d, ST_WALL_HITS);
    if (my_hits) atomicAdd(&d.counters->wall_hits, my_hits);
    if (surf) surf_flush(acc, surf, my_hits != 0);
}

WallView make_walls(mz_ctx* c, const mz_grid1d* g, const mz_walls1d* w)
{
    WallView W;
    W.L = g->L;
    W.min_x = g->min_x;
    W.max_x = g->max_x;
    W.inv_dx = g->inv_dx;
    W.trig = c->d_trig;
    wall_bits(W);
    for (int b = 0; b < 2; ++b) {
        for (int q = 0; q < MZ_MAX_SPECIES; ++q) W.vsq[b][q] = w->reflection_v_sq[b][q];
        W.acc[b] = w->accommodation[b];
        for (int k = 0; k < 3; ++k) W.wv[b][k] = w->v[b][k];
    }
    return W;
}

}  // namespace

void launch_convect_count(mz_domain* d, int s, const mz_grid1d* g, const mz_walls1d* w, double dt,
                          const uint32_t* step_ptr, const long long* hw_dev, const int* abort, double* surf)
{
    mz_ctx* c = d->ctx;
    const WallView W = make_walls(c, g, w);
    DomainView v = make_view(d);
    const int blocks =
        (int)std::max<int64_t>(1, std::min<int64_t>(div_up(d->sp[s].capacity, 256), (int64_t)c->num_sms * 8));
    MZ_LAUNCH(c, "convect", k_convect_count, blocks, 256, 0, v, s, hw_dev, W, dt, step_ptr, abort, surf);
}

void launch_convect(mz_domain* d, int s, const mz_grid1d* g, const mz_walls1d* w, double dt, uint64_t step,
                    int32_t flags, double* surf)
{
    mz_ctx* c = d->ctx;
    SpeciesHost& S = d->sp[s];
    if (S.hw <= 0) return;
    const WallView W = make_walls(c, g, w);
    DomainView v = make_view(d);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(S.hw, 256), (int64_t)c->num_sms * 8));
    MZ_LAUNCH(c, "convect", k_convect, blocks, 256, 0, v, s, S.hw, W, dt, (uint32_t)step,
              (flags & MZ_CONVECT_COMPUTE_CELL) ? 1 : 0, surf);
}
