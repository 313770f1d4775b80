// Fused time step: the loop body of simulations/1D/couette_benchmarking.jl:58-85
// (ntc_equal_weight! -> convect_particles! -> sort_particles! ->
// compute_props_sorted! -> avg_props!) and of the 0-D drivers (README.md:91-106:
// ntc! for every species pair -> compute_props!).
//
// One warp owns 32 / G cells for the whole step (G: lanes per cell in NTC,
// ntc_group_width).  With a 1-D grid, one step is
//   scan (per species)    : counts accumulated by the previous step -> indexer
//                           (two passes, launch_scan_cells)
//   scatter (per species) : slot tickets per destination cell
//   k_cell                : sort the cell's segment and gather its particles
//                           (A -> B, the only full read+write of particle
//                           data), compute props of the sorted state, then
//                           NTC and convection of the next step on the
//                           gathered particles, new cell ids and counts.
// so particle data crosses HBM once per step (112 B per particle).  0-D steps
// run k_cell in place (no sort).  The RNG step index lives in device memory
// and is advanced by the last block of k_cell, so a whole step is captured
// once in a CUDA graph and replayed.
#include "cell_ops.cuh"
#include "mz_host.h"
#include "ntc_block.cuh"
#include "sortnet.cuh"

#include <algorithm>

using namespace mz;

namespace {

struct PropsPtrs {
    double *np, *n, *v, *T;
};

struct StepArgs {
    WallView W;
    double dt;
    int dims;          // 0 or 1
    int gather;        // sort segment + gather A -> B
    int props;         // compute props of the (gathered) state
    int physics;       // NTC + convection of the next step
    int advance;       // the last block advances the RNG step index
    int has_inst, has_avg;
    PropsPtrs inst, avg;
    double inv_navg;
    int64_t avg_start; // averaging when (step index of the props) - step0 >= avg_start
    uint64_t step0;
    int props_lag;     // props describe the state after step (step - props_lag)
    uint32_t* step_ptr;   // RNG step of the NTC / convection done by this launch
    unsigned int* done;   // last-block counter
    unsigned int* next;   // next cell to hand out (cells are taken CPW at a time)
    int4* hitq;           // particles that reach a wall: {slot, cell, position in cell, species}
    unsigned int* hit_n;  // entries in hitq
    unsigned int* hit_done;  // last-block counter of k_wall_hits
    unsigned int* big_next;  // next cell k_ntc_big examines
    unsigned int* big_done;  // last-block counter of k_ntc_big
    unsigned int join_blocks;  // k_cell and k_ntc_big overlap: their blocks together on `done` (0 = not)
    unsigned int hitq_cap;
    int32_t big_cell;     // cells with at least this many particles collide in k_ntc_big
    double* surf;         // wall sums of this step [species][2][11], or nullptr
    double* surf_avg;     // their average, or nullptr
    double surf_factor[MZ_MAX_SPECIES];  // mass / dt per species (surface_props_scale!)
    const int* abort;     // variable-weight step: nonzero = the step was abandoned (do nothing), or nullptr
    // producer / consumer launch (k_cell_ws): gathered cells are published
    // in ready[c] with the launch's tag (*epoch + 1, unique per launch)
    int* ready;
    unsigned int* epoch;
    unsigned int* cons_next;  // next cell for the consumer warps
    int producer_warps;       // warps per block that gather
};

// release store / acquire load of a publication word (GPU scope)
__device__ __forceinline__ void st_release(int* p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire(const int* p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// bounded wait until *p == v: back-off sleeps, at most ~2^24 tries (seconds);
// false when it gave up
__device__ __forceinline__ bool wait_for(const int* p, int v)
{
    for (int k = 0; k < (1 << 24); ++k) {
        if (ld_acquire(p) == v) return true;
        __nanosleep(k < 64 ? 32 : 256);
    }
    return false;
}

// cells of the per-warp destination histogram of k_cell (48 KB per block)
constexpr int CELL_WINDOW = 1536;
constexpr size_t CELL_SMEM = (size_t)8 * CELL_WINDOW * sizeof(int32_t);

__device__ __forceinline__ void write_props(const StepArgs& a, int64_t ix, const CellMoments& r, int32_t np,
                                            uint32_t step)
{
    if (a.has_inst) {
        a.inst.np[ix] = (double)np;
        a.inst.n[ix] = r.n;
        a.inst.v[3 * ix + 0] = r.ux;
        a.inst.v[3 * ix + 1] = r.uy;
        a.inst.v[3 * ix + 2] = r.uz;
        a.inst.T[ix] = r.T;
    }
    if (a.has_avg && (int64_t)(step - a.props_lag) - (int64_t)a.step0 >= a.avg_start) {
        const double f = a.inv_navg;
        a.avg.np[ix] = fma((double)np, f, a.avg.np[ix]);
        a.avg.n[ix] = fma(r.n, f, a.avg.n[ix]);
        a.avg.v[3 * ix + 0] = fma(r.ux, f, a.avg.v[3 * ix + 0]);
        a.avg.v[3 * ix + 1] = fma(r.uy, f, a.avg.v[3 * ix + 1]);
        a.avg.v[3 * ix + 2] = fma(r.uz, f, a.avg.v[3 * ix + 2]);
        a.avg.T[ix] = fma(r.T, f, a.avg.T[ix]);
    }
}

// A warp takes CPW = 32 / G consecutive cells at a time.  Sorting, gathering,
// props and convection run cell by cell on the whole warp; NTC runs on all CPW
// cells at once, one group of G lanes per cell.  The grid is resident (one
// wave) and hands out cells through an atomic counter, so no partial last wave
// idles the GPU.
// MODE 0: the phases the launch's flags select; MODE 1: sort + gather + props
// only (no NTC or convection code, so fewer registers and more resident
// warps for this memory-bound part); MODE 2: NTC + convection in place only.
// WS (k_cell_ws): MODE 1 warps gather through their shared-memory stage and
// publish every gathered cell; MODE 2 warps take cells from their own
// counter, wait for the cells' publication (acquire) and run NTC + convection
// on the gathered buffer B.
template <int G, int MODE, bool WS = false, bool BIG = false>
__device__ __forceinline__ void cell_body(const DomainView& d, const StepArgs& a, int32_t* cell_hist,
                                          double2* stage = nullptr, int32_t* sortbuf = nullptr)
{
    constexpr int CPW = 32 / G;
    const bool gather_on = MODE == 1 ? true : (MODE == 2 ? false : a.gather != 0);
    const bool physics_on = MODE == 1 ? false : (MODE == 2 ? true : a.physics != 0);
    const bool onB = gather_on || (WS && MODE == 2);  // the physics works on the gathered buffer
    const uint32_t step = *a.step_ptr;
    const int tag = WS ? (int)(*a.epoch + 1u) : 0;
    const int lane = threadIdx.x & 31;
    int32_t* wh = cell_hist + (threadIdx.x >> 5) * CELL_WINDOW;
    if (MODE != 1) {
        for (int bin = lane; bin < CELL_WINDOW; bin += 32) wh[bin] = 0;
        __syncwarp();
    }
    const WarpGroup<G> grp;
    const int gi = lane / G;
    const int ns = d.n_species;
    unsigned long long cand = 0, accd = 0, hits = 0;
    bool cap = false;
    const bool abandoned = a.abort && *a.abort;
    // a resident grid; warps take the next CPW cells until none are left
    for (;;) {
        if (abandoned) break;
        unsigned int t = 0;
        if (lane == 0) t = atomicAdd((WS && MODE == 2) ? a.cons_next : a.next, (unsigned)CPW);
        const int c0 = (int)__shfl_sync(0xFFFFFFFFu, t, 0);
        if (c0 >= d.n_cells) break;
        const int nq = min(CPW, d.n_cells - c0);
        if (WS && MODE == 2) {
            // wait until the producers have published these cells
            bool ok = true;
            if (lane < nq) ok = wait_for(a.ready + c0 + lane, tag);
            if (!ok) set_status(d, ST_TIMEOUT);
            __syncwarp();
            __threadfence();
        }
        // sort + gather (A -> B), then 1-D props of the freshly sorted state
        // (the gather accumulates the first props pass)
        for (int s = 0; s < ns; ++s) {
            const SpeciesView& S = d.sp[s];
            // the physics-only mode never computes props (in the side-by-side
            // launch the gathering warps do)
            const bool props1 = MODE != 2 && a.props && a.props_lag == 1;
            double mn = 0.0, msx = 0.0, msy = 0.0, msz = 0.0;
            if (gather_on) {
                for (int q = 0; q < nq; ++q) {
                    const Indexer p = S.ind[c0 + q];
                    const Sums4 t = (WS && MODE == 1) ? sort_gather_segment_staged(S, c0 + q, p.start1, p.n1, stage)
                                                      : sort_gather_segment<BIG, MODE == 1 && !WS>(S, c0 + q, p.start1,
                                                                                            p.n1, sortbuf);
                    if (props1) props_pass1_into_lane(t.n, t.sx, t.sy, t.sz, q, mn, msx, msy, msz);
                }
                __syncwarp();
                if (props1) {
                    const CellMoments r = props_cells_finish(S.B, S.ind, c0, nq, S.mass, mn, msx, msy, msz);
                    if (lane < nq)
                        write_props(a, (int64_t)(c0 + lane) + (int64_t)d.n_cells * s, r, S.ind[c0 + lane].n1, step);
                }
            } else if (props1) {
                const CellMoments r = props_cells(S.A, S.ind, c0, nq, S.mass);
                if (lane < nq)
                    write_props(a, (int64_t)(c0 + lane) + (int64_t)d.n_cells * s, r, S.ind[c0 + lane].n1, step);
            }
        }
        if (WS && MODE == 1) {
            // publish: every lane's stores of these cells before the flag
            __threadfence();
            __syncwarp();
            if (lane < nq) st_release(a.ready + c0 + lane, tag);
            continue;
        }
        __syncwarp();
        if (!physics_on && !(a.props && a.props_lag == 0)) continue;
        // ntc_equal_weight! for every pair in the reference's order, one
        // group per cell
        const int c = c0 + gi;
        bool big = false;
        if (gi < nq) {
            int32_t tot = 0;
            for (int s = 0; s < ns; ++s) tot += d.sp[s].ind[c].n1;
            big = tot >= a.big_cell;
        }
        if (physics_on && gi < nq && !big) {
            const uint64_t seed = cell_seed(d, c);
            const uint32_t rid = cell_rid(d, c), stp = cell_step(d, c, step);
            const double V = d.cell_V[c];
            for (int s2 = 0; s2 < ns; ++s2) {
                for (int s1 = s2; s1 < ns; ++s1) {
                    const bool single = s1 == s2;
                    const int cfi = s1 + ns * s2;
                    const SpeciesView& S1 = d.sp[s1];
                    const SpeciesView& S2 = d.sp[s2];
                    Indexer q1 = S1.ind[c], q2 = S2.ind[c];
                    CollisionFactors cf = d.cf[(size_t)cfi * d.n_cells + c];
                    const uint32_t pc = (uint32_t)(s1 * ns + s2);
                    const int32_t ncoll = ntc_ncoll(d, cf, single, q1.n1, q2.n1, a.dt, V, seed, pc, stp, rid);
                    NtcResult R;
                    R.smax = cf.smax;
                    R.perf = R.eqw = R.nsp1 = R.nsp2 = 0;
                    if (ncoll > 0)
                        R = ntc_cell<true, G>(d, d.inter[cfi], single, c, ncoll, cf.smax, onB ? S1.B : S1.A,
                                              onB ? S2.B : S2.A, q1, q2, nullptr, nullptr, nullptr, nullptr, 0, 0,
                                              0.0, seed, pc, stp, rid);
                    if (grp.rank == 0) {
                        cand += ncoll;
                        accd += R.perf;
                        cf.smax = R.smax;
                        cf.n_coll_performed = R.perf;
                        cf.n_eq_w_coll_performed = R.eqw;
                        d.cf[(size_t)cfi * d.n_cells + c] = cf;
                    }
                }
            }
        }
        __syncwarp();
        // 0-D: compute_props! after the collisions of this step
        if (a.props && a.props_lag == 0) {
            // large cells get their props in k_ntc_big
            const unsigned skip = __ballot_sync(0xFFFFFFFFu, grp.rank == 0 && big) >> 0;
            unsigned skipq = 0u;
            for (int q = 0; q < nq; ++q)
                if ((skip >> (q * G)) & 1u) skipq |= 1u << q;
            for (int s = 0; s < ns; ++s) {
                const SpeciesView& S = d.sp[s];
                const CellMoments r = props_cells(gather_on ? S.B : S.A, S.ind, c0, nq, S.mass, skipq);
                if (lane < nq && !((skipq >> lane) & 1u))
                    write_props(a, (int64_t)(c0 + lane) + (int64_t)d.n_cells * s, r, S.ind[c0 + lane].n1, step);
            }
        }
        if (a.dims != 1 || !physics_on) continue;
        // convect_particles! + get_cell for the next sort.  Destination counts
        // go to a per-warp histogram over a window of cells around the warp's
        // cells, flushed with one atomic per non-empty cell (consecutive
        // addresses); destinations outside the window count directly.
        const int kb = c0 + CPW / 2 - CELL_WINDOW / 2;
        for (int s = 0; s < ns; ++s) {
            const SpeciesView& S = d.sp[s];
            const Cols& Q = onB ? S.B : S.A;
            for (int q = 0; q < nq; ++q) {
                const int cq = c0 + q;
                const uint64_t seed = cell_seed(d, cq);
                const uint32_t rid = cell_rid(d, cq), stp = cell_step(d, cq, step);
                const Indexer p = S.ind[cq];
                const int32_t n1 = p.n1, st1 = p.start1;
                // each row's position and velocity are loaded one row ahead,
                // before the current row's stores (other particles)
                double x_next = 0.0, vx_next = 0.0;
                if (lane < n1) {
                    x_next = Q.pos[(int64_t)st1 + lane].x;
                    vx_next = Q.wv[(int64_t)st1 + lane].vx;
                }
                for (int j0 = 0; j0 < n1; j0 += 32) {
                    const int j = j0 + lane;
                    const bool in = j < n1;
                    const int64_t qq = (int64_t)st1 + j;
                    const double x_row = x_next, vx_row = vx_next;
                    if (j + 32 < n1) {
                        x_next = Q.pos[qq + 32].x;
                        vx_next = Q.wv[qq + 32].vx;
                    }
                    int32_t key = 0;
                    bool counted = false, hit = false;
                    if (in) {
                        double x = x_row;
                        const double xn = fma(vx_row, a.dt, x);
                        if (move_free(a.W, xn, x)) {
                            Q.pos[qq].x = x;
                            key = cell_of(d, x, a.W.inv_dx);
                            S.key[qq] = key;
                            counted = true;
                        } else {
                            hit = true;
                        }
                    }
                    // particles that reach a wall finish in k_wall_hits, packed
                    // into full warps; a full queue falls back to this warp
                    const unsigned hm = __ballot_sync(0xFFFFFFFFu, hit);
                    if (hm) {
                        const int leader = __ffs(hm) - 1;
                        unsigned base = 0;
                        if (lane == leader) base = atomicAdd(a.hit_n, (unsigned)__popc(hm));
                        base = __shfl_sync(0xFFFFFFFFu, base, leader);
                        const unsigned k = base + __popc(hm & lanemask_lt());
                        if (hit && k < a.hitq_cap) {
                            a.hitq[k] = make_int4((int)qq, cq, j, s);
                        } else if (hit) {
                            Stream rs;
                            rs.init(seed, TAG_CONVECT, (uint32_t)s, stp, rid, (uint32_t)j);
                            const PV r = Q.wv[qq];
                            double x = Q.pos[qq].x, vx = r.vx, vy = r.vy, vz = r.vz;
                            SurfAcc one = {};
                            hits += convect_walls(rs, a.W, s, x, vx, vy, vz, a.dt, cap, a.surf ? &one : nullptr, r.w);
                            if (a.surf)
                                for (int e = 0; e < 2; ++e)
                                    for (int k = 0; k < SURF_Q; ++k)
                                        if (one.q[e][k] != 0.0)
                                            atomicAdd(&a.surf[((size_t)s * 2 + e) * SURF_Q + k], one.q[e][k]);
                            Q.wv[qq] = PV{r.w, vx, vy, vz};
                            Q.pos[qq].x = x;
                            key = cell_of(d, x, a.W.inv_dx);
                            S.key[qq] = key;
                            counted = true;
                        }
                    }
                    if (counted) {
                        const int bin = key - kb;
                        if ((unsigned)bin < (unsigned)CELL_WINDOW)
                            atomicAdd(&wh[bin], 1);
                        else
                            atomicAdd(&S.counts[key], 1);
                    }
                }
            }
            __syncwarp();
            for (int bin = lane; bin < CELL_WINDOW; bin += 32) {
                const int v = wh[bin];
                if (v) {
                    atomicAdd(&S.counts[kb + bin], v);
                    wh[bin] = 0;
                }
            }
            __syncwarp();
        }
    }
    if (cap) set_status(d, ST_WALL_HITS);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_xor_sync(0xFFFFFFFFu, cand, o);
        accd += __shfl_xor_sync(0xFFFFFFFFu, accd, o);
        hits += __shfl_xor_sync(0xFFFFFFFFu, hits, o);
    }
    if (lane == 0 && (cand | accd | hits)) {
        atomicAdd(&d.counters->candidates, cand);
        atomicAdd(&d.counters->accepted, accd);
        atomicAdd(&d.counters->wall_hits, hits);
    }
    // the last block to finish advances the RNG step for the next launch
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(a.done, 1u);
        if (prev == (a.join_blocks ? a.join_blocks : gridDim.x) - 1) {
            *a.done = 0;
            *a.next = 0;
            if (a.join_blocks) *a.big_next = 0;
            if (WS) {
                *a.cons_next = 0;
                *a.epoch = (unsigned)tag;
            }
            if (a.advance) *a.step_ptr = step + 1;
            __threadfence();
        }
    }
}


template <int G>
__global__ void __launch_bounds__(256, 2) k_cell(DomainView d, StepArgs a)
{
    extern __shared__ int32_t cell_hist[];  // CELL_WINDOW bins per warp
    cell_body<G, 0>(d, a, cell_hist);
}

// One cell per warp: the gather's random reads fetch whole 128-byte lines,
// and a line's other records (neighbouring particles of the old order) are
// gathered into nearby cells soon after; with one cell in flight per warp the
// lines in flight fit in L2 and are reused there (four cells per warp keep
// twice the L2 in flight and miss).
__global__ void __launch_bounds__(256, 3) k_cell_gather(DomainView d, StepArgs a)
{
    cell_body<32, 1>(d, a, nullptr);
}

// The same for the variable-weight step, whose cells often hold more than
// 1,024 particles: two warps per block with registers for 64-row sorts
// (segments up to 2,048) and a shared-memory buffer each for larger ones.
constexpr int GB_THREADS = 64;
constexpr size_t GB_SMEM = (size_t)(GB_THREADS / 32) * SORT_SMEM_KEYS * sizeof(int32_t);
__global__ void __launch_bounds__(GB_THREADS) k_cell_gather_big(DomainView d, StepArgs a)
{
    extern __shared__ int32_t sortbuf[];
    cell_body<32, 1, false, true>(d, a, nullptr, nullptr, sortbuf + (size_t)(threadIdx.x >> 5) * SORT_SMEM_KEYS);
}

template <int G>
__global__ void __launch_bounds__(256, 2) k_cell_physics(DomainView d, StepArgs a)
{
    extern __shared__ int32_t cell_hist[];  // CELL_WINDOW bins per warp
    cell_body<G, 2>(d, a, cell_hist);
}

// The 1-D step in one launch with the two halves of the two-launch form side
// by side, one block of WS_THREADS per SM: the first producer_warps warps sort,
// gather and compute props cell by cell and publish each gathered cell; their
// gathers go through a shared-memory stage of STAGE_ROWS records per warp, so
// a few warps keep a whole cell's reads in flight each (the memory-bound
// half needs bytes in flight, not warps).  The other warps take cells in
// groups of 32 / G, wait for them and run NTC + convection on them
// (FP64-bound) while their records are still in L2.  Producers never wait,
// so every cell a consumer waits for is gathered by a running producer.
constexpr int WS_THREADS = 512, WS_PRODUCERS = 4;
constexpr size_t WS_SMEM = (size_t)(WS_THREADS / 32) * CELL_WINDOW * sizeof(int32_t) +
                           (size_t)WS_PRODUCERS * STAGE_ROWS * 4 * sizeof(double2);

template <int G>
__global__ void __launch_bounds__(WS_THREADS, 1) k_cell_ws(DomainView d, StepArgs a)
{
    extern __shared__ int32_t cell_hist[];  // CELL_WINDOW bins per warp, then the producers' stages
    const int w = (int)(threadIdx.x >> 5);
    if (w < a.producer_warps) {
        double2* stage = reinterpret_cast<double2*>(cell_hist + (WS_THREADS / 32) * CELL_WINDOW) +
                         (size_t)w * STAGE_ROWS * 4;
        cell_body<32, 1, true>(d, a, cell_hist, stage);
    } else {
        cell_body<G, 2, true>(d, a, cell_hist);
    }
}

__global__ void k_set_step(uint32_t* step, uint32_t value) { *step = value; }

// ntc_equal_weight! and the 0-D compute_props! of the cells with at least
// a.big_cell particles, one block per cell (ntc_cell_block, props_cell_block);
// k_cell skips these cells' collisions and props.  Blocks take the next large
// cell from a counter when they finish one, so a block never holds several
// large cells while others idle (the last block resets the counter).
__global__ void __launch_bounds__(NTC_BLOCK, 2) k_ntc_big(DomainView d, StepArgs a)
{
    __shared__ NtcBlockShared sh;
    __shared__ double red[4 * (NTC_BLOCK / 32)];
    __shared__ int next_cell;
    const uint32_t step = *a.step_ptr;
    const int ns = d.n_species;
    unsigned long long cand = 0, accd = 0;
    for (;;) {
        if (threadIdx.x == 0) {
            // skip small cells here, without block barriers
            int c = (int)atomicAdd(a.big_next, 1u);
            for (; c < d.n_cells; c = (int)atomicAdd(a.big_next, 1u)) {
                int32_t tot = 0;
                for (int s = 0; s < ns; ++s) tot += d.sp[s].ind[c].n1;
                if (tot >= a.big_cell) break;
            }
            next_cell = c;
        }
        __syncthreads();
        const int c = next_cell;
        __syncthreads();
        if (c >= d.n_cells) break;
        const uint64_t seed = cell_seed(d, c);
        const uint32_t rid = cell_rid(d, c), stp = cell_step(d, c, step);
        const double V = d.cell_V[c];
        for (int s2 = 0; s2 < ns && a.physics; ++s2) {
            for (int s1 = s2; s1 < ns; ++s1) {
                const bool single = s1 == s2;
                const int cfi = s1 + ns * s2;
                const SpeciesView& S1 = d.sp[s1];
                const SpeciesView& S2 = d.sp[s2];
                const Indexer q1 = S1.ind[c], q2 = S2.ind[c];
                CollisionFactors cf = d.cf[(size_t)cfi * d.n_cells + c];
                const uint32_t pc = (uint32_t)(s1 * ns + s2);
                const int32_t ncoll = ntc_ncoll(d, cf, single, q1.n1, q2.n1, a.dt, V, seed, pc, stp, rid);
                NtcResult R;
                R.smax = cf.smax;
                R.perf = R.eqw = R.nsp1 = R.nsp2 = 0;
                if (ncoll > 0)
                    R = ntc_cell_block(sh, d.inter[cfi], single, ncoll, cf.smax, a.gather ? S1.B : S1.A,
                                       a.gather ? S2.B : S2.A, q1, q2, d.trig, seed, pc, stp, rid);
                if (threadIdx.x == 0) {
                    cand += ncoll;
                    accd += R.perf;
                    cf.smax = R.smax;
                    cf.n_coll_performed = R.perf;
                    cf.n_eq_w_coll_performed = R.eqw;
                    d.cf[(size_t)cfi * d.n_cells + c] = cf;
                }
                __syncthreads();
            }
        }
        // 0-D: compute_props! of the cell after its collisions
        if (a.props && a.props_lag == 0) {
            for (int s = 0; s < ns; ++s) {
                const SpeciesView& S = d.sp[s];
                const Indexer p = S.ind[c];
                const CellMoments r = props_cell_block(a.gather ? S.B : S.A, p, S.mass, red);
                if (threadIdx.x == 0) write_props(a, (int64_t)c + (int64_t)d.n_cells * s, r, p.n1, step);
            }
        }
    }
    if (threadIdx.x == 0) {
        if (cand | accd) {
            atomicAdd(&d.counters->candidates, cand);
            atomicAdd(&d.counters->accepted, accd);
        }
        __threadfence();
        if (a.join_blocks) {
            // overlapping k_cell: the last block of either launch resets both
            // cell counters and advances the RNG step
            if (atomicAdd(a.done, 1u) == a.join_blocks - 1) {
                *a.done = 0;
                *a.next = 0;
                *a.big_next = 0;
                if (a.advance) *a.step_ptr = step + 1;
                __threadfence();
            }
        } else if (atomicAdd(a.big_done, 1u) == gridDim.x - 1) {
            *a.big_next = 0;
            *a.big_done = 0;
            __threadfence();
        }
    }
}

// The wall-hit loop of convect_particles! (convection_1D.jl:22-46) for the
// particles k_cell queued, one thread each, with the particle's own stream:
// the same arithmetic and draws as in k_cell, but the FP64 work of diffuse
// reflections (log, sqrt, sine and cosine) runs on full warps.
__global__ void __launch_bounds__(256) k_wall_hits(DomainView d, StepArgs a)
{
    const uint32_t step = *a.step_ptr - 1;  // k_cell advanced it
    const unsigned n = min(*a.hit_n, a.hitq_cap);
    unsigned long long hits = 0;
    bool cap = false;
    SurfAcc acc[MZ_MAX_SPECIES > 1 ? 1 : 1] = {};
    int acc_s = -1;  // species of this thread's sums (flushed when it changes)
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int4 h = a.hitq[i];
        const int64_t qq = h.x;
        const int c = h.y, j = h.z, s = h.w;
        const SpeciesView& S = d.sp[s];
        const Cols& Q = a.gather ? S.B : S.A;
        Stream rs;
        rs.init(cell_seed(d, c), TAG_CONVECT, (uint32_t)s, cell_step(d, c, step), cell_rid(d, c), (uint32_t)j);
        const PV r = Q.wv[qq];
        double x = Q.pos[qq].x, vx = r.vx, vy = r.vy, vz = r.vz;
        SurfAcc* sa = nullptr;
        if (a.surf) {
            if (acc_s >= 0 && acc_s != s) {
                // another species: add this thread's sums directly
                for (int e = 0; e < 2; ++e)
                    for (int k = 0; k < SURF_Q; ++k)
                        if (acc[0].q[e][k] != 0.0) atomicAdd(&a.surf[((size_t)acc_s * 2 + e) * SURF_Q + k], acc[0].q[e][k]);
                acc[0] = SurfAcc{};
            }
            acc_s = s;
            sa = &acc[0];
        }
        hits += convect_walls(rs, a.W, s, x, vx, vy, vz, a.dt, cap, sa, r.w);
        Q.wv[qq] = PV{r.w, vx, vy, vz};
        Q.pos[qq].x = x;
        const int32_t key = cell_of(d, x, a.W.inv_dx);
        S.key[qq] = key;
        atomicAdd(&S.counts[key], 1);
    }
    if (cap) set_status(d, ST_WALL_HITS);
    if (a.surf) {
        // block sums per species of the last sums each thread holds
        for (int s = 0; s < d.n_species; ++s)
            surf_flush(acc_s == s ? acc[0] : SurfAcc{}, a.surf + (size_t)s * 2 * SURF_Q, acc_s == s);
    }
    hits = __reduce_add_sync(0xFFFFFFFFu, (unsigned)hits);
    if ((threadIdx.x & 31) == 0 && hits) atomicAdd(&d.counters->wall_hits, hits);
    // the last block empties the queue for the next step
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(a.hit_done, 1u);
        if (prev == gridDim.x - 1) {
            *a.hit_done = 0;
            *a.hit_n = 0;
            __threadfence();
        }
    }
}

// Tickets of the counting sort: each block takes tiles of SCATTER_TILE
// consecutive slots; slots whose destination lies within SCATTER_WINDOW cells
// of the tile's middle cell take a rank from a shared-memory histogram, and
// each non-empty destination then reserves its run of the cell's segment
// with one global atomic (consecutive addresses).  Other slots take a ticket
// directly.  The order inside a segment is arbitrary; k_cell sorts it.
constexpr int SCATTER_TILE = 4096, SCATTER_WINDOW = 2048;

// surface_props_scale! of the step's wall sums, then avg_props! into the
// average from avg_start on (the convection of RNG step `step`)
__global__ void k_surf_finish(StepArgs a, int ns)
{
    if (a.abort && *a.abort) return;
    const uint32_t step = *a.step_ptr - 1;  // k_cell advanced it
    const bool averaging = a.surf_avg && (int64_t)step - (int64_t)a.step0 >= a.avg_start;
    for (int i = threadIdx.x; i < ns * 2 * SURF_Q; i += blockDim.x) {
        const int s = i / (2 * SURF_Q);
        double v = a.surf[i];
        if (i % SURF_Q != 0) v *= a.surf_factor[s];
        a.surf[i] = v;
        if (averaging) a.surf_avg[i] = fma(v, a.inv_navg, a.surf_avg[i]);
    }
}

// n_dev (variable-weight step): the slot count from device memory, and slots
// whose cell is -1 (dead) take no ticket
__global__ void __launch_bounds__(256, 4) k_step_scatter(DomainView d, int s, int64_t n, const long long* n_dev,
                                                         const int* abort)
{
    __shared__ int32_t hist[SCATTER_WINDOW];
    constexpr int PER = SCATTER_TILE / 256;
    const SpeciesView& S = d.sp[s];
    if (abort && *abort) return;
    if (n_dev) n = *n_dev;
    for (int64_t t0 = (int64_t)blockIdx.x * SCATTER_TILE; t0 < n; t0 += (int64_t)gridDim.x * SCATTER_TILE) {
        const int64_t t1 = min(n, t0 + (int64_t)SCATTER_TILE);
        // every load of the tile first, so that they are in flight together
        // (and across the barrier below)
        int32_t key[PER], rank[PER];
#pragma unroll
        for (int r = 0; r < PER; ++r) {
            const int64_t slot = t0 + threadIdx.x + 256 * r;
            const bool in = slot < t1;
            key[r] = in ? S.key[slot] : 0;
            rank[r] = in && (!n_dev || S.cell[slot] >= 0) ? 0 : -1;
        }
        const int32_t cmid = S.cell[(t0 + t1 - 1) / 2];
        const int kb = (cmid >= 0 ? cmid : S.key[(t0 + t1 - 1) / 2]) - SCATTER_WINDOW / 2;
        for (int b = threadIdx.x; b < SCATTER_WINDOW; b += blockDim.x) hist[b] = 0;
        __syncthreads();
#pragma unroll
        for (int r = 0; r < PER; ++r) {
            const int64_t slot = t0 + threadIdx.x + 256 * r;
            const bool live = rank[r] == 0;
            rank[r] = -1;
            if (live) {
                const int32_t k = key[r];
                const int b = k - kb;
                if ((unsigned)b < (unsigned)SCATTER_WINDOW) {
                    rank[r] = atomicAdd(&hist[b], 1);
                } else {
                    const int32_t pos = S.ind[k].start1 + atomicAdd(&S.fill[k], 1);
                    S.idx[pos] = (int32_t)slot;
                }
            }
        }
        __syncthreads();
        for (int b = threadIdx.x; b < SCATTER_WINDOW; b += blockDim.x) {
            const int cnt = hist[b];
            if (cnt) hist[b] = S.ind[kb + b].start1 + atomicAdd(&S.fill[kb + b], cnt);
        }
        __syncthreads();
#pragma unroll
        for (int r = 0; r < PER; ++r)
            if (rank[r] >= 0) S.idx[hist[key[r] - kb] + rank[r]] = (int32_t)(t0 + threadIdx.x + 256 * r);
        __syncthreads();
    }
}

// ------------------------------------------------ variable-weight step
// The loop body of simulations/1D/couette_varweight_octree.jl:85-135 (and of
// the 0-D variable-weight drivers, test_bkw_varweight_octree.jl): per cell
// ntc! with splitting (collision_ntc.jl:338-380), then
// merge_octree_N2_based! of the cells above a threshold, then convection
// and the sort with compute_props_sorted!.  Every kernel reads the RNG step
// and the slot counts from device memory, so a step is captured once in a
// CUDA graph with no host synchronisation.  The first kernel computes every
// cell's candidate count (compute_n_coll_single_species,
// collision_ntc.jl:173-184), which bounds its splits; the scan of those
// counts reserves each cell's split region after the used slots, and the
// step is abandoned right there -- before any particle changes -- when the
// reservation would pass the storage capacity or a cell could outgrow the
// merge scratch (the host grows both and resumes the step).

// n_coll of every cell and the split reservation res[c] = n_coll; cells that
// may be merged must fit the merge scratch (nmax particles)
__global__ void k_vw_prepare(DomainView d, int s, double dt, const uint32_t* step_ptr, VwDev* vw, int32_t* res,
                             int merging, int64_t threshold, int64_t nmax)
{
    if (vw->abort) return;
    const uint32_t step = *step_ptr;
    const SpeciesView& S = d.sp[s];
    const int ns = d.n_species;
    const int cfi = s + ns * s;
    const uint32_t pc = (uint32_t)(s * ns + s);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < d.n_cells; c += gridDim.x * blockDim.x) {
        const Indexer p = S.ind[c];
        const int64_t n = (int64_t)p.n1 + p.n2;
        CollisionFactors& cf = d.cf[(size_t)cfi * d.n_cells + c];
        const int32_t nc = ntc_ncoll(d, cf, true, n, n, dt, d.cell_V[c], cell_seed(d, c), pc,
                                     cell_step(d, c, step), cell_rid(d, c));
        res[c] = nc;
        if (merging && n + nc > threshold && n + nc > nmax) {
            atomicMax(&vw->need_cell, (long long)(n + nc));
            atomicOr(&vw->abort, VW_SCRATCH);
        }
    }
}

// after the scan of the reservations (total in sp.need): the slots in use
// after the splits, or the step is abandoned for capacity
__global__ void k_vw_check(VwDev* vw, int s, long long capacity)
{
    if (vw->abort) return;
    VwSpecies& q = vw->sp[s];
    const long long need = q.hw + q.need;
    q.need = need;
    if (need > capacity)
        vw->abort |= VW_CAPACITY;
    else
        q.hw_split = need;
}

// ntc! of every cell, one group of G lanes per cell; split particles go to
// the cell's reserved region [base[c], base[c] + res[c]), whose unused slots
// become dead (as k_ntc does for the standalone entry point)
template <int G>
__global__ void __launch_bounds__(256) k_vw_ntc(DomainView d, int s, double dw_tol, const uint32_t* step_ptr,
                                                const int* abort, const int32_t* base, const int32_t* res)
{
    if (*abort) return;
    const uint32_t step = *step_ptr;
    const SpeciesView& S = d.sp[s];
    const int ns = d.n_species;
    const int cfi = s + ns * s;
    const uint32_t pc = (uint32_t)(s * ns + s);
    const Interaction I = d.inter[cfi];
    const WarpGroup<G> grp;
    const int ngroups = (gridDim.x * blockDim.x) / G;
    unsigned long long cand = 0, accd = 0, spl = 0;
    for (int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) / G); c < d.n_cells; c += ngroups) {
        CollisionFactors* cfp = &d.cf[(size_t)cfi * d.n_cells + c];
        const int32_t ncoll = cfp->n_coll;
        if (ncoll <= 0) continue;
        Indexer p1 = S.ind[c];
        const int32_t b1 = base[c];
        const NtcResult R = ntc_cell_split<G, NTC_SPLIT_VERSIONS>(d, I, c, ncoll, cfp->smax, S.A, p1, S.cell, S.key,
                                                                  b1, dw_tol, cell_seed(d, c), pc,
                                                                  cell_step(d, c, step), cell_rid(d, c));
        if (grp.rank == 0) {
            cfp->smax = R.smax;
            cfp->n_coll_performed = R.perf;
            cfp->n_eq_w_coll_performed = R.eqw;
            cfp->n_split = R.nsp1;
            S.ind[c] = p1;
            cand += ncoll;
            accd += R.perf;
            spl += R.nsp1;
        }
        const int32_t r1 = res[c];
        for (int32_t q = R.nsp1 + grp.rank; q < r1; q += G) S.cell[b1 + q] = -1;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        cand += __shfl_xor_sync(0xFFFFFFFFu, cand, o);
        accd += __shfl_xor_sync(0xFFFFFFFFu, accd, o);
        spl += __shfl_xor_sync(0xFFFFFFFFu, spl, o);
    }
    if ((threadIdx.x & 31) == 0 && cand) {
        atomicAdd(&d.counters->candidates, cand);
        atomicAdd(&d.counters->accepted, accd);
        atomicAdd(&d.counters->splits, spl);
    }
}

// 0-D: every live slot stays in its cell; counting it there lets the sort
// machinery compact the cells (squash_pia!) for the props
__global__ void k_vw_keep(DomainView d, int s, const long long* hw_dev, const int* abort)
{
    if (*abort) return;
    const SpeciesView& S = d.sp[s];
    const int64_t hw = *hw_dev;
    const int lane = threadIdx.x & 31;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x + threadIdx.x - lane; base < hw;
         base += (int64_t)gridDim.x * blockDim.x) {
        const int64_t slot = base + lane;
        const int32_t c = slot < hw ? S.cell[slot] : -1;
        const unsigned m = __ballot_sync(0xFFFFFFFFu, c >= 0);
        if (c >= 0) {
            S.key[slot] = c;
            warp_agg_add(S.counts, c, m);
        }
    }
}

__global__ void k_vw_advance(uint32_t* step, const int* abort)
{
    if (!*abort) *step += 1u;
}

}  // namespace

// launch arguments every fused step shares: walls, props and averaging,
// surface sampling, the device step index and cell counters
static StepArgs step_args(mz_domain* d, const mz_step_plan* plan, mz_props* inst, mz_props* avg)
{
    mz_ctx* c = d->ctx;
    StepArgs a;
    memset(&a, 0, sizeof a);
    a.W.L = plan->grid.L;
    a.W.min_x = plan->grid.min_x;
    a.W.max_x = plan->grid.max_x;
    a.W.inv_dx = plan->grid.inv_dx;
    a.W.trig = c->d_trig;
    wall_bits(a.W);
    for (int b = 0; b < 2; ++b) {
        for (int q = 0; q < MZ_MAX_SPECIES; ++q) a.W.vsq[b][q] = plan->walls.reflection_v_sq[b][q];
        a.W.acc[b] = plan->walls.accommodation[b];
        for (int k = 0; k < 3; ++k) a.W.wv[b][k] = plan->walls.v[b][k];
    }
    a.dt = plan->dt;
    a.dims = plan->dims;
    if (plan->dims == 1 && d->step_surf) {
        a.surf = d->step_surf->acc;
        a.surf_avg = d->step_surf_avg ? d->step_surf_avg->acc : nullptr;
        for (int s = 0; s < d->ns; ++s) a.surf_factor[s] = d->mass[s] / plan->dt;
    }
    // block-per-cell collisions for large 0-D cells (the 1-D step keeps every
    // cell's phases in one warp)
    {
        int32_t big = plan->big_cell != 0 ? plan->big_cell : (d->tuned_big != 0 ? d->tuned_big : 2048);
        a.big_cell = plan->dims == 0 && big > 0 ? big : INT_MAX;
    }
    a.has_inst = inst != nullptr;
    a.has_avg = avg != nullptr && plan->avg_start > 0;
    if (inst) a.inst = PropsPtrs{inst->np, inst->n, inst->v, inst->T};
    if (avg) a.avg = PropsPtrs{avg->np, avg->n, avg->v, avg->T};
    a.inv_navg = plan->n_avg > 0 ? 1.0 / (double)plan->n_avg : 0.0;
    a.avg_start = plan->avg_start;
    a.step0 = plan->step0;
    a.props_lag = plan->dims == 1 ? 1 : 0;
    a.step_ptr = d->d_step;
    a.done = d->d_done;
    a.next = d->d_done + 1;
    a.hit_n = d->d_done + 2;
    a.hit_done = d->d_done + 3;
    a.big_next = d->d_done + 4;
    a.big_done = d->d_done + 5;
    return a;
}

static void ensure_step_words(mz_domain* d)
{
    if (!d->d_step) {
        MZ_CK(cudaMalloc(&d->d_step, sizeof(uint32_t)));
        MZ_CK(cudaMalloc(&d->d_done, 8 * sizeof(unsigned int)));
        MZ_CK(cudaMemsetAsync(d->d_done, 0, 8 * sizeof(unsigned int), d->ctx->stream));
    }
}

static void launch_step_vw(mz_domain* d, const mz_step_plan* plan, int64_t n_steps, mz_props* inst, mz_props* avg);

void launch_step(mz_domain* d, const mz_step_plan* plan, int64_t n_steps, mz_props* inst, mz_props* avg)
{
    mz_ctx* c = d->ctx;
    if (n_steps <= 0) return;
    if (!plan->equal_weight) {
        launch_step_vw(d, plan, n_steps, inst, avg);
        return;
    }
    // the 1-D step's sort runs over slots [0, n_total): close gaps first; the
    // 0-D step works on each cell's group-1 list in place, so only split
    // particles in group 2 need a compaction
    for (int s = 0; s < d->ns; ++s)
        if (plan->dims == 1 || d->sp[s].group2) launch_compact(d, s);
    ensure_step_words(d);
    const uint32_t first = (uint32_t)(plan->step0 + 1);
    // a one-thread kernel, not a copy from pageable host memory: such a copy
    // waits for the stream to drain, and the host would then launch the next
    // step's kernels on an idle GPU
    MZ_LAUNCH(c, "step_set_index", k_set_step, 1, 1, 0, d->d_step, first);
    StepArgs a = step_args(d, plan, inst, avg);
    if (plan->dims == 1) {
        // wall-hit queue: a fraction of the particles (or the plan's size);
        // overflow is handled inline
        int64_t n_all = 0;
        for (int s = 0; s < d->ns; ++s) n_all += d->sp[s].n_total;
        const int64_t want =
            plan->hit_queue_capacity > 0 ? plan->hit_queue_capacity : std::max<int64_t>(4096, n_all / 16);
        if (want > d->hitq_cap) {
            cudaFree(d->d_hitq);
            d->d_hitq = nullptr;
            d->hitq_cap = 0;
            MZ_CK(cudaMalloc(&d->d_hitq, want * sizeof(int4)));
            d->hitq_cap = want;
        }
        a.hitq = static_cast<int4*>(d->d_hitq);
        a.hitq_cap = (unsigned)std::min<int64_t>(std::min(want, d->hitq_cap), 0x7FFFFFFF);
    }
    const bool want_props = plan->props && (inst || a.has_avg);
    const bool split = plan->dims == 1 && (plan->launches == 2 || (plan->launches == 0 && d->tuned_split == 1));
    // one launch with gathering and physics warps side by side (k_cell_ws)
    const bool ws = plan->dims == 1 && (plan->launches == 3 || (plan->launches == 0 && d->tuned_split == 2));
    if (ws) {
        if (!d->d_ready) {
            MZ_CK(cudaMalloc(&d->d_ready, d->n_cells * sizeof(int)));
            MZ_CK(cudaMemsetAsync(d->d_ready, 0, d->n_cells * sizeof(int), c->stream));
        }
        a.ready = d->d_ready;
        a.cons_next = d->d_done + 6;
        a.epoch = d->d_done + 7;
        a.producer_warps = WS_PRODUCERS;
    }
    const int G = d->tuned_lanes ? d->tuned_lanes : ntc_group_width(d->n_cells);
    using KCell = void (*)(DomainView, StepArgs);
    const KCell kern_full = G == 8 ? k_cell<8> : (G == 16 ? k_cell<16> : k_cell<32>);
    const KCell kern_phys = G == 8 ? k_cell_physics<8> : (G == 16 ? k_cell_physics<16> : k_cell_physics<32>);
    const KCell kern_ws = G == 8 ? k_cell_ws<8> : (G == 16 ? k_cell_ws<16> : k_cell_ws<32>);
    // a resident grid: as many blocks as fit at once, no more than the cells need
    auto resident = [&](KCell k, size_t smem, int cpw) {
        int per_sm = 0;
        MZ_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, smem));
        return (int)std::max<int64_t>(
            1, std::min<int64_t>(div_up(d->n_cells, 8 * cpw), (int64_t)c->num_sms * std::max(per_sm, 1)));
    };
    const int blocks_full = resident(kern_full, CELL_SMEM, 32 / G);
    const int blocks_phys = plan->dims == 1 ? resident(kern_phys, CELL_SMEM, 32 / G) : 0;
    const int blocks_gather = plan->dims == 1 ? resident(k_cell_gather, 0, 1) : 0;
    int blocks_ws = 0;
    if (ws) {
        MZ_CK(cudaFuncSetAttribute(kern_ws, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WS_SMEM));
        int per_sm = 0;
        MZ_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern_ws, WS_THREADS, WS_SMEM));
        MZ_REQUIRE(per_sm >= 1, "step: the side-by-side launch does not fit on an SM");
        blocks_ws = (int)std::max<int64_t>(
            1, std::min<int64_t>(div_up(d->n_cells, 8), (int64_t)c->num_sms * per_sm));
    }

    auto cell_launch = [&](int gather, int props, int physics, int advance = 1) {
        StepArgs b = a;
        b.gather = gather;
        b.props = props;
        b.physics = physics;
        b.advance = advance;
        DomainView v = make_view(d);
        // distinct names: the full step (gather + props + physics) is the one
        // the roofline is quoted on
        const char* name = !gather ? "step_cell_inplace" : (physics ? "step_cell" : "step_cell_final");
        // 0-D: the large cells' blocks (k_ntc_big) and the warp-per-cell
        // launch work on disjoint cells and run side by side (fork / join
        // through events, also inside a graph capture); the last block of
        // the two advances the step
        const bool big_launch = (physics || props) && b.big_cell < INT_MAX;
        const bool overlap = big_launch && a.dims == 0;
        if (overlap) {
            b.join_blocks = (unsigned)(c->num_sms * 2 + blocks_full);
            MZ_CK(cudaEventRecord(c->ev_fork, c->stream));
            MZ_CK(cudaStreamWaitEvent(c->side, c->ev_fork, 0));
            {
                struct OnSide {  // MZ_LAUNCH targets c->stream: the side stream for this launch
                    mz_ctx* c;
                    cudaStream_t main;
                    ~OnSide() { c->stream = main; }
                } on_side{c, c->stream};
                c->stream = c->side;
                MZ_LAUNCH(c, "step_ntc_big", k_ntc_big, c->num_sms * 2, NTC_BLOCK, 0, v, b);
            }
            MZ_CK(cudaEventRecord(c->ev_join, c->side));
        } else if (big_launch) {
            MZ_LAUNCH(c, "step_ntc_big", k_ntc_big, c->num_sms * 2, NTC_BLOCK, 0, v, b);
        }
        if (physics && b.surf)
            MZ_CK(cudaMemsetAsync(b.surf, 0, (size_t)d->ns * 2 * SURF_Q * sizeof(double), c->stream));
        // 1-D launches that only sort + gather + props, or only collide and
        // convect, take the kernels compiled for that part alone
        if (a.dims == 1 && gather && physics && ws)
            MZ_LAUNCH(c, name, kern_ws, blocks_ws, WS_THREADS, WS_SMEM, v, b);
        else if (a.dims == 1 && gather && !physics)
            MZ_LAUNCH(c, name, k_cell_gather, blocks_gather, 256, 0, v, b);
        else if (a.dims == 1 && !gather && !props && physics)
            MZ_LAUNCH(c, name, kern_phys, blocks_phys, 256, CELL_SMEM, v, b);
        else
            MZ_LAUNCH(c, name, kern_full, blocks_full, 256, CELL_SMEM, v, b);
        if (overlap) MZ_CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
        if (physics && a.dims == 1) MZ_LAUNCH(c, "step_wall_hits", k_wall_hits, c->num_sms * 2, 256, 0, v, b);
        if (physics && b.surf) MZ_LAUNCH(c, "step_surf", k_surf_finish, 1, 128, 0, b, d->ns);
    };
    // one sort of every species from the keys k_cell wrote, gather in k_cell
    auto sort_launch = [&](int props, int physics) {
        DomainView v = make_view(d);
        for (int s = 0; s < d->ns; ++s) {
            SpeciesHost& S = d->sp[s];
            launch_scan_cells(d, S.counts, S.ind, S.fill, d->d_scalar + s, true, nullptr, 0);
            const int sb = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(S.n_total, SCATTER_TILE), (int64_t)c->num_sms * 8));
            MZ_LAUNCH(c, "step_scatter", k_step_scatter, sb, 256, 0, v, s, S.n_total, (const long long*)nullptr,
                      (const int*)nullptr);
        }
        if (split && physics) {
            // gather + props, then NTC + convection in place on the sorted
            // state: each launch keeps less data in flight between its reads
            cell_launch(1, props, 0, 0);
            for (int s = 0; s < d->ns; ++s) d->sp[s].cur ^= 1;  // B holds the sorted state
            cell_launch(0, 0, physics);
        } else {
            cell_launch(1, props, physics);
            for (int s = 0; s < d->ns; ++s) d->sp[s].cur ^= 1;  // B holds the sorted state
        }
    };

    const bool graph = plan->use_graph != 0;
    if (plan->dims == 1) {
        // the first step's NTC + convection run in place on the sorted state
        cell_launch(0, 0, plan->collide);
        const int64_t middle = n_steps - 1;
        if (middle > 0) {
            if (graph && middle > 1) {
                // capture one step (scan, scatter, k_cell) and replay it; the
                // two buffers alternate, so the graph covers two steps
                cudaGraph_t g = nullptr;
                cudaGraphExec_t ge = nullptr;
                const int64_t launches0 = c->launches;
                MZ_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
                sort_launch(want_props, plan->collide);
                sort_launch(want_props, plan->collide);
                MZ_CK(cudaStreamEndCapture(c->stream, &g));
                const int64_t per_graph = c->launches - launches0;
                MZ_CK(cudaGraphInstantiate(&ge, g, 0));
                const int64_t pairs = middle / 2;
                for (int64_t i = 0; i < pairs; ++i) MZ_CK(cudaGraphLaunch(ge, c->stream));
                c->launches += per_graph * (pairs - 1);
                if (middle % 2) sort_launch(want_props, plan->collide);
                // the captured launches swapped `cur` twice: buffers are back
                // in the order the replays leave them
                MZ_CK(cudaGraphExecDestroy(ge));
                MZ_CK(cudaGraphDestroy(g));
            } else {
                for (int64_t t = 0; t < middle; ++t) sort_launch(want_props, plan->collide);
            }
        }
        // final sort + props of the last step, no further physics
        sort_launch(want_props, 0);
    } else {
        for (int64_t t = 0; t < n_steps; ++t) cell_launch(0, want_props, plan->collide);
    }
    if (plan->dims == 1)
        for (int s = 0; s < d->ns; ++s) {
            d->sp[s].hw = d->sp[s].n_total;
            d->sp[s].compact = true;
        }
}

// The variable-weight loop with the standalone kernels, step by step (a
// mixture: each pair's splits change the cells the next pair draws from, so
// no reservation can be made for the whole step before it starts).
static void launch_step_vw_sequence(mz_domain* d, const mz_step_plan* plan, int64_t n_steps, mz_props* inst,
                                    mz_props* avg)
{
    mz_ctx* c = d->ctx;
    const bool want_props = plan->props && (inst || (avg && plan->avg_start > 0));
    mz_props* p = inst;
    mz_props* own = nullptr;
    if (want_props && !p) {
        MZ_REQUIRE(mz_props_create(d, 0, nullptr, 300.0, avg->ndens, &own) == MZ_OK, "mz_step: props");
        p = own;
    }
    const int64_t m = d->n_cells * d->ns;
    for (int64_t k = 1; k <= n_steps; ++k) {
        const uint64_t step = plan->step0 + (uint64_t)k;
        if (plan->collide)
            for (int s2 = 0; s2 < d->ns; ++s2)
                for (int s1 = s2; s1 < d->ns; ++s1)
                    launch_ntc(d, s1, s2, plan->dt, 0, d->n_cells, step, 0, plan->dw_tol);
        for (int s = 0; s < d->ns; ++s) {
            if (plan->merge_threshold > 0)
                launch_merge(d, s, 0, d->n_cells, plan->merge_threshold, plan->merge_target, &plan->octree,
                             plan->dims == 1 ? &plan->grid : nullptr, step, nullptr);
            if (plan->dims == 1) {
                launch_convect(d, s, &plan->grid, &plan->walls, plan->dt, step, 0);
                launch_sort(d, s, &plan->grid, nullptr);
            } else {
                launch_compact(d, s);
            }
        }
        if (want_props) {
            launch_props(d, p, plan->dims == 1 ? MZ_PROPS_SORTED : MZ_PROPS_ALL);
            if (avg && plan->avg_start > 0 && k >= plan->avg_start) {
                const double inv = 1.0 / (double)plan->n_avg;
                launch_avg(c, avg->np, p->np, m, inv);
                launch_avg(c, avg->n, p->n, m, inv);
                launch_avg(c, avg->v, p->v, 3 * m, inv);
                launch_avg(c, avg->T, p->T, m, inv);
            }
        }
    }
    if (own) mz_props_destroy(own);
}

// Variable-weight steps of one species, device-resident and graph-replayed
// (the kernels k_vw_prepare .. k_cell_gather above).  A step abandoned for
// capacity or merge scratch leaves the state of the step before; the host
// reads how many steps finished, grows what was short and runs the rest, so
// the result equals an uninterrupted run.
static void launch_step_vw(mz_domain* d, const mz_step_plan* plan, int64_t n_steps, mz_props* inst, mz_props* avg)
{
    mz_ctx* c = d->ctx;
    MZ_REQUIRE(plan->dims == 0 || plan->dims == 1, "mz_step: dims must be 0 or 1");
    const bool merging = plan->merge_threshold > 0;
    if (merging) MZ_REQUIRE(plan->merge_target >= 1, "mz_step: merge_target must be at least 1");
    if (d->ns != 1) {
        launch_step_vw_sequence(d, plan, n_steps, inst, avg);
        return;
    }
    const int s = 0;
    SpeciesHost& S = d->sp[s];
    launch_compact(d, s);
    ensure_step_words(d);
    if (!d->d_vw) {
        MZ_CK(cudaMalloc(&d->d_vw, sizeof(VwDev)));
        MZ_CK(cudaMallocHost(&d->h_vw, sizeof(VwDev)));
    }
    if (merging) {
        d->vw_nmax = std::max<int64_t>(d->vw_nmax, std::max<int64_t>(2 * plan->merge_threshold,
                                                                     plan->merge_threshold + 2048));
        merge_fused_reserve(d, d->vw_nmax, plan->merge_target, &plan->octree);
    }
    MZ_CK(cudaMemsetAsync(S.counts, 0, (d->n_cells + 1) * sizeof(int32_t), c->stream));
    const bool want_props = plan->props && (inst || (avg && plan->avg_start > 0));
    // lanes per cell of the splitting NTC (the autotuner's choice, else 8):
    // a batch ends at its first split, so a cell's batches hold ~2-3
    // candidates and narrow groups let one FP64 instruction serve several
    // cells; with few cells, one-warp blocks spread the warps over every SM
    const int G = plan->split_lanes ? plan->split_lanes : (d->tuned_vw_lanes ? d->tuned_vw_lanes : 32);
    MZ_REQUIRE(G == 8 || G == 16 || G == 32, "mz_step: split_lanes must be 0, 8, 16 or 32");
    using KNtc = void (*)(DomainView, int, double, const uint32_t*, const int*, const int32_t*, const int32_t*);
    const KNtc kntc = G == 8 ? k_vw_ntc<8> : (G == 16 ? k_vw_ntc<16> : k_vw_ntc<32>);
    const int cblocks = (int)std::max<int64_t>(1, std::min<int64_t>(div_up(d->n_cells, 256), (int64_t)c->num_sms * 8));
    const int64_t ntc_warps = div_up(d->n_cells, 32 / G);
    const int ntc_threads = ntc_warps >= 8 * (int64_t)c->num_sms ? 256 : 32;
    const int nblocks = (int)std::max<int64_t>(
        1, std::min<int64_t>(div_up(ntc_warps * 32, ntc_threads), (int64_t)c->num_sms * 16 * (256 / ntc_threads)));
    // the gather takes one cell per warp, in two-warp blocks (which also
    // spread few cells over every SM) with their segments' sort buffers
    const int gthreads = GB_THREADS;
    int per_sm = 0;
    MZ_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_cell_gather_big, gthreads, GB_SMEM));
    const int gblocks = (int)std::max<int64_t>(
        1, std::min<int64_t>(div_up(d->n_cells, gthreads / 32), (int64_t)c->num_sms * std::max(per_sm, 1)));
    VwDev* V = d->d_vw;
    const int* abort = &V->abort;

    int64_t done = 0;
    while (done < n_steps) {
        memset(d->h_vw, 0, sizeof(VwDev));
        d->h_vw->sp[s].hw = S.n_total;
        MZ_CK(cudaMemcpyAsync(d->d_vw, d->h_vw, sizeof(VwDev), cudaMemcpyHostToDevice, c->stream));
        const uint32_t first = (uint32_t)(plan->step0 + 1 + (uint64_t)done);
        MZ_LAUNCH(c, "step_set_index", k_set_step, 1, 1, 0, d->d_step, first);
        StepArgs a = step_args(d, plan, inst, avg);
        a.abort = abort;
        a.props_lag = 1;  // the gather runs after the step index advanced
        const int cur0 = S.cur;
        const int64_t sblocks = std::max<int64_t>(
            1, std::min<int64_t>(div_up(S.capacity, SCATTER_TILE), (int64_t)c->num_sms * 8));
        auto one_step = [&]() {
            DomainView v = make_view(d);
            if (plan->collide) {
                // n_coll and split reservations, then the reservations' bases
                // after the used slots and the capacity check
                MZ_LAUNCH(c, "vw_prepare", k_vw_prepare, cblocks, 256, 0, v, s, plan->dt, d->d_step, V, S.fill,
                          merging ? 1 : 0, plan->merge_threshold, d->vw_nmax);
                launch_scan_cells(d, S.fill, S.ind, S.fill, reinterpret_cast<int64_t*>(&V->sp[s].need), false,
                                  S.work, 0, nullptr, &V->sp[s].hw, abort);
            } else {
                MZ_CK(cudaMemsetAsync(&V->sp[s].need, 0, sizeof(long long), c->stream));
            }
            MZ_LAUNCH(c, "vw_check", k_vw_check, 1, 1, 0, V, s, (long long)S.capacity);
            if (plan->collide)
                MZ_LAUNCH(c, "vw_ntc", kntc, nblocks, ntc_threads, 0, v, s, plan->dw_tol, d->d_step, abort, S.work,
                          S.fill);
            if (merging)
                launch_merge_fused(d, s, plan->merge_threshold, plan->merge_target, &plan->octree,
                                   plan->dims == 1 ? &plan->grid : nullptr, d->d_step, abort, d->vw_nmax,
                                   V->sp[s].merge);
            if (plan->dims == 1) {
                if (a.surf)
                    MZ_CK(cudaMemsetAsync(a.surf, 0, (size_t)d->ns * 2 * SURF_Q * sizeof(double), c->stream));
                launch_convect_count(d, s, &plan->grid, &plan->walls, plan->dt, d->d_step, &V->sp[s].hw_split,
                                     abort, a.surf);
            } else {
                MZ_LAUNCH(c, "vw_keep", k_vw_keep, (int)sblocks, 256, 0, v, s, &V->sp[s].hw_split, abort);
            }
            MZ_LAUNCH(c, "vw_advance", k_vw_advance, 1, 1, 0, d->d_step, abort);
            if (a.surf) MZ_LAUNCH(c, "step_surf", k_surf_finish, 1, 128, 0, a, d->ns);
            // sort_particles! over the used slots (dead ones skipped) and
            // compute_props_sorted! of the sorted state
            launch_scan_cells(d, S.counts, S.ind, S.fill, reinterpret_cast<int64_t*>(&V->sp[s].hw), true, nullptr, 0,
                              nullptr, nullptr, abort);
            MZ_LAUNCH(c, "step_scatter", k_step_scatter, (int)sblocks, 256, 0, v, s, (int64_t)0, &V->sp[s].hw_split,
                      abort);
            StepArgs b = a;
            b.gather = 1;
            b.props = want_props ? 1 : 0;
            b.physics = 0;
            b.advance = 0;
            MZ_LAUNCH(c, "step_cell_final", k_cell_gather_big, gblocks, gthreads, GB_SMEM, v, b);
            S.cur ^= 1;
        };
        const int64_t todo = n_steps - done;
        if (plan->use_graph && todo > 2) {
            // two steps per graph: the buffers alternate
            cudaGraph_t g = nullptr;
            cudaGraphExec_t ge = nullptr;
            const int64_t launches0 = c->launches;
            MZ_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            one_step();
            one_step();
            MZ_CK(cudaStreamEndCapture(c->stream, &g));
            const int64_t per_graph = c->launches - launches0;
            MZ_CK(cudaGraphInstantiate(&ge, g, 0));
            const int64_t pairs = todo / 2;
            for (int64_t i = 0; i < pairs; ++i) MZ_CK(cudaGraphLaunch(ge, c->stream));
            c->launches += per_graph * (pairs - 1);
            if (todo % 2) one_step();
            MZ_CK(cudaGraphExecDestroy(ge));
            MZ_CK(cudaGraphDestroy(g));
        } else {
            for (int64_t t = 0; t < todo; ++t) one_step();
        }
        MZ_CK(cudaMemcpyAsync(d->h_vw, d->d_vw, sizeof(VwDev), cudaMemcpyDeviceToHost, c->stream));
        MZ_CK(cudaMemcpyAsync(d->h_scalar + 7, d->d_step, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
        MZ_CK(cudaStreamSynchronize(c->stream));
        uint32_t now = 0;
        memcpy(&now, d->h_scalar + 7, sizeof now);
        const int64_t completed = (int64_t)(now - first);
        MZ_REQUIRE(completed >= 0 && completed <= todo, "mz_step: step index out of range");
        S.cur = cur0 ^ (int)(completed & 1);
        S.n_total = S.hw = d->h_vw->sp[s].hw;
        S.compact = true;
        S.group2 = false;
        done += completed;
        const int why = d->h_vw->abort;
        if (!why) {
            MZ_REQUIRE(completed == todo, "mz_step: steps missing");
            break;
        }
        if (why & VW_CAPACITY) {
            const int64_t need = d->h_vw->sp[s].need;
            reserve_species(d, s, need + need / 8 + 1024);
        }
        if (why & VW_SCRATCH) {
            d->vw_nmax = d->h_vw->need_cell + d->h_vw->need_cell / 4 + 256;
            merge_fused_reserve(d, d->vw_nmax, plan->merge_target, &plan->octree);
        }
    }
}

// Time every mapping of the fused step on real steps of the simulation (the
// mapping changes no result, so the trial steps are ordinary steps) and keep
// the fastest for later mz_step calls: lanes per cell in the warp-group NTC
// and, for 0-D cells, the particle count from which a cell collides one block
// per cell.
void autotune_step(mz_domain* d, const mz_step_plan* plan, int64_t trial_steps, int32_t* lanes_out, int32_t* big_out)
{
    mz_ctx* c = d->ctx;
    const int32_t lanes_c[3] = {8, 16, 32};
    const int32_t big_c[4] = {512, 2048, 8192, -1};
    // the second choice: the block-per-cell threshold (0-D) or the fused
    // against the two-launch step (1-D)
    // a variable-weight plan has only the lanes per cell of its splitting NTC
    const bool vw = !plan->equal_weight;
    const int nb = vw ? 1 : (plan->dims == 0 ? 4 : 3);
    const int nconf = 3 * nb;
    mz_step_plan p = *plan;
    p.big_cell = 0;
    p.launches = 0;
    p.split_lanes = 0;
    std::vector<float> total(nconf, 0.0f);
    uint64_t step = plan->step0;
    cudaEvent_t e0, e1;
    MZ_CK(cudaEventCreate(&e0));
    MZ_CK(cudaEventCreate(&e1));
    auto apply = [&](int k) {
        if (vw) {
            d->tuned_vw_lanes = lanes_c[k / nb];
            return;
        }
        d->tuned_lanes = lanes_c[k / nb];
        d->tuned_big = plan->dims == 0 ? big_c[k % nb] : -1;
        d->tuned_split = plan->dims == 0 ? 0 : k % nb;
    };
    // a variable-weight plan's lanes change only its splitting NTC, while the
    // merge's share of a step varies from step to step: its trials time the
    // NTC launches alone (direct launches, each bracketed by events)
    const bool kt_was = c->kernel_timing;
    if (vw) {
        p.use_graph = 0;
        c->kernel_timing = true;
    }
    auto ntc_ms = [&]() {
        c->resolve_timings();
        for (const KernelTiming& t : c->timings)
            if (t.name == "vw_ntc") return t.total_ms;
        return 0.0;
    };
    // two rounds, the second in reverse order, and a configuration's time is
    // the sum of its two: the step time drifts as the simulation evolves (the
    // collision-rate estimate adapts), and the reversal cancels a linear drift
    for (int round = 0; round < 2; ++round)
        for (int i = 0; i < nconf; ++i) {
            const int k = round == 0 ? i : nconf - 1 - i;
            apply(k);
            p.step0 = step;
            const double before = vw ? ntc_ms() : 0.0;
            MZ_CK(cudaEventRecord(e0, c->stream));
            launch_step(d, &p, trial_steps, nullptr, nullptr);
            MZ_CK(cudaEventRecord(e1, c->stream));
            MZ_CK(cudaEventSynchronize(e1));
            float ms = 0.0f;
            MZ_CK(cudaEventElapsedTime(&ms, e0, e1));
            if (vw) ms = (float)(ntc_ms() - before);
            step += (uint64_t)trial_steps;
            total[k] += ms;
        }
    if (vw && !kt_was) {
        // the trials' timings were the tuner's own
        c->resolve_timings();
        c->timings.clear();
    }
    c->kernel_timing = kt_was;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    apply((int)(std::min_element(total.begin(), total.end()) - total.begin()));
    if (lanes_out) *lanes_out = vw ? d->tuned_vw_lanes : d->tuned_lanes;
    if (big_out) *big_out = vw ? 0 : (plan->dims == 0 ? d->tuned_big : d->tuned_split);
}
