// Host-side state behind the C ABI (include/merzgpu.h).
#pragma once

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/merzgpu.h"
#include "mz_internal.cuh"

struct MzError : std::runtime_error {
    int code;
    MzError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define MZ_CK(call)                                                                                    \
    do {                                                                                               \
        cudaError_t _e = (call);                                                                       \
        if (_e != cudaSuccess)                                                                         \
            throw MzError(MZ_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));              \
    } while (0)

#define MZ_REQUIRE(cond, msg)                                                                          \
    do {                                                                                               \
        if (!(cond)) throw MzError(MZ_E_ARG, msg);                                                     \
    } while (0)

struct KernelTiming {
    std::string name;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pending;
    double total_ms = 0.0;
    int64_t launches = 0;
};

struct mz_ctx_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;  // a second stream for launches that overlap the main one
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::string last_error;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    void* flush_buf = nullptr;
    size_t flush_bytes = 0;
    bool kernel_timing = false;
    std::vector<KernelTiming> timings;
    std::vector<cudaEvent_t> event_pool;
    int64_t launches = 0;
    int num_sms = 0;
    double2* d_trig = nullptr;  // sector table of sincos_2pi_u52 (2 x TRIG_SECTORS)

    cudaEvent_t get_event();
    // bracket a launch with events when kernel timing is on; returns slot or -1
    int timer_begin(const char* name, cudaEvent_t* start);
    void timer_end(int slot, cudaEvent_t start);
    void resolve_timings();
    bool capturing() const;
};

struct SpeciesHost {
    int64_t capacity = 0;
    int64_t hw = 0;        // high water: slots [0, hw) in use (live or dead)
    int64_t n_total = 0;   // live particles
    bool compact = true;   // every cell's list lies in group 1 and no dead slot below hw
    bool group2 = false;   // some cell may hold group-2 (split) particles
    mz::PV* wv[2] = {nullptr, nullptr};   // [buffer A/B] weight + velocity records
    mz::PX* pos[2] = {nullptr, nullptr};  // [buffer A/B] position records
    int cur = 0;           // which buffer is A
    int32_t* cell[2] = {nullptr, nullptr};  // [A/B] owner cell per slot
    int32_t* key = nullptr;
    int32_t* idx = nullptr;
    int32_t* counts = nullptr;  // n_cells + 1
    int32_t* fill = nullptr;
    int32_t* work = nullptr;    // n_cells + 1 scratch (reservations / bases)
    mz::Indexer* ind = nullptr;
};

// Device words of the fused variable-weight step.  Slot counts live on the
// device there (the host learns them at the end of the call); a step that
// would overflow the particle storage or the merge scratch is abandoned
// before it changes any particle: `abort` is set, every later kernel of the
// call returns at once, and the host grows the storage and resumes.
enum : int { VW_CAPACITY = 1, VW_SCRATCH = 2 };
struct VwSpecies {
    long long hw;        // slots in use at the start of a step (the live count after the last sort)
    long long hw_split;  // slots in use after this step's split reservations
    long long need;      // slots the abandoned step needed (VW_CAPACITY)
    long long merge[4];  // merge kernels: particles deleted, cells merged, cell counters of the warp and block forms
};
struct VwDev {
    VwSpecies sp[MZ_MAX_SPECIES];
    int abort;             // VW_* reasons
    int pad;
    long long need_cell;   // particles of the largest cell the merge scratch must hold (VW_SCRATCH)
};

struct mz_domain_s {
    mz_ctx* ctx = nullptr;
    int64_t n_cells = 0;
    int32_t ns = 0;
    SpeciesHost sp[MZ_MAX_SPECIES];
    double mass[MZ_MAX_SPECIES] = {0};
    mz::Interaction inter[MZ_MAX_SPECIES * MZ_MAX_SPECIES];
    double* d_V = nullptr;
    uint64_t* d_cell_seed = nullptr;
    uint32_t* d_cell_rid = nullptr;
    uint32_t* d_cell_step = nullptr;
    mz::CollisionFactors* d_cf = nullptr;
    mz::Counters* d_counters = nullptr;
    int* d_status = nullptr;
    int64_t* d_scalar = nullptr;   // small device scratch (totals), 16 entries
    int64_t* d_tile_sums = nullptr;  // per-tile totals of the cell scans
    int64_t* h_scalar = nullptr;   // pinned mirror
    uint64_t seed = 1234;
    // octree scratch (allocated on demand)
    void* d_merge_scratch = nullptr;
    size_t merge_scratch_bytes = 0;
    // property sets created on this domain (freed with it)
    std::vector<mz_props*> props;
    std::vector<mz_surf_props*> surf;
    // surface sampling of the fused 1-D step (mz_step_set_surface)
    mz_surf_props* step_surf = nullptr;
    mz_surf_props* step_surf_avg = nullptr;
    // fused step: RNG step index and last-block counter
    uint32_t* d_step = nullptr;
    unsigned int* d_done = nullptr;  // fused step: {last block, next cell, wall hits queued, wall last block, next big cell, big last block, next consumer cell, launch epoch}
    void* d_hitq = nullptr;          // fused step: wall-hit queue (int4 entries)
    int64_t hitq_cap = 0;
    // fused-step mapping chosen by mz_step_autotune (0: the default rules)
    int32_t tuned_lanes = 0;    // lanes per cell in k_cell's NTC (8, 16, 32)
    int32_t tuned_vw_lanes = 0; // lanes per cell of the variable-weight step's splitting NTC (8, 16, 32)
    int32_t tuned_big = 0;      // 0-D block-per-cell threshold (-1: never)
    int32_t tuned_split = 0;    // 1-D: 1 = gather + props and NTC + convection in two launches,
                                // 2 = one launch with gathering and physics warps side by side
    int* d_ready = nullptr;     // per-cell publication words of that launch
    struct mz_slab_scratch* slab = nullptr;  // slab exchange scratch (slab.cu)
    // fused variable-weight step
    VwDev* d_vw = nullptr;
    VwDev* h_vw = nullptr;      // pinned mirror
    int64_t vw_nmax = 0;        // particles per cell the merge scratch holds
};

// SurfProps of a domain's 1-D walls (surface_props.jl:22-67): device sums
// [species][element][11] in the order np, flux_incident, flux_reflected,
// force xyz, normal_pressure, shear_pressure xyz, kinetic_energy_flux
struct mz_surf_props_s {
    mz_domain* dom = nullptr;
    double* acc = nullptr;  // n_species * 2 * 11
};

struct mz_props_s {
    mz_domain* dom = nullptr;
    int32_t n_moments = 0;
    int32_t powers[16] = {0};
    double Tref = 300.0;
    int32_t ndens = 0;
    // device arrays in Merzbild's column-major layouts
    double* np = nullptr;       // n_cells * ns
    double* n = nullptr;        // n_cells * ns
    double* v = nullptr;        // 3 * n_cells * ns
    double* T = nullptr;        // n_cells * ns
    double* moments = nullptr;  // n_moments * n_cells * ns
    double lpa[MZ_MAX_SPECIES] = {0};
    void* snapshot = nullptr;   // asynchronous read-back state (snapshot.cu)
};

// ---------------------------------------------------------------- helpers
mz::DomainView make_view(mz_domain* d);
void ensure_compact(mz_domain* d, int s);
void swap_buffers(mz_domain* d, int s);
void check_status(mz_domain* d);
void free_props_snapshot(mz_props* p);
// last-error text of a context, and the try / catch that turns MzError and
// other exceptions into a status code at every C entry point
void set_err(const mz_ctx* c, const std::string& m);
#define API_TRY try {
#define API_CATCH(ctxp)                                                                                \
    }                                                                                                  \
    catch (MzError & e)                                                                                \
    {                                                                                                  \
        set_err(ctxp, e.what());                                                                       \
        return e.code;                                                                                 \
    }                                                                                                  \
    catch (std::exception & e)                                                                         \
    {                                                                                                  \
        set_err(ctxp, e.what());                                                                       \
        return MZ_E_ARG;                                                                               \
    }                                                                                                  \
    return MZ_OK;

int64_t div_up(int64_t a, int64_t b);

// launchers (one per translation unit)
void launch_sort(mz_domain* d, int s, const mz_grid1d* grid, int64_t* out_index);
void launch_compact(mz_domain* d, int s);
// exclusive scan of per-cell counts (or of n1 + n2 of nlocal_from): cell
// starts into base_out and/or a fresh group-1 indexer (write_indexer, which
// also zeroes fill and counts), the total into total_out
void launch_scan_cells(mz_domain* d, int32_t* counts, mz::Indexer* ind, int32_t* fill, int64_t* total_out,
                       bool write_indexer, int32_t* base_out, int64_t base_offset,
                       const mz::Indexer* nlocal_from = nullptr, const long long* base_offset_dev = nullptr,
                       const int* abort = nullptr);
void launch_ntc(mz_domain* d, int s1, int s2, double dt, int64_t cb, int64_t ce, uint64_t step, int32_t flags,
                double dw_tol);
void launch_props(mz_domain* d, mz_props* p, int32_t mode);
// surf: this species' 2 x 11 surface sums, or nullptr
void launch_convect(mz_domain* d, int s, const mz_grid1d* g, const mz_walls1d* w, double dt, uint64_t step,
                    int32_t flags, double* surf = nullptr);
void launch_sample_cells(mz_domain* d, int s, const int64_t* counts_host, const int32_t* counts_dev,
                         const double* T3, const double* T3_all, const double* Fnum, double span, const double* box6,
                         int32_t distribution, uint64_t step, const double* v0 = nullptr,
                         const double* v0_all = nullptr);
void launch_sample_grid(mz_domain* d, int s, const mz_grid1d* g, double ndens, double T, double Fnum, uint64_t step,
                        const double* v0_all = nullptr);
void launch_merge(mz_domain* d, int s, int64_t cb, int64_t ce, int64_t threshold, int64_t target,
                  const mz_octree_params* prm, const mz_grid1d* grid, uint64_t step, int64_t* n_merged);
// merging inside the fused step: no host synchronisation; the step index and
// an abort word come from device memory, scratch is reserved beforehand for
// cells of up to nmax particles; words3 = {deleted, merged, cell counters of the warp and block forms}
int merge_fused_warps(mz_domain* d);
void merge_fused_reserve(mz_domain* d, int64_t nmax, int64_t target, const mz_octree_params* prm);
void launch_merge_fused(mz_domain* d, int s, int64_t threshold, int64_t target, const mz_octree_params* prm,
                        const mz_grid1d* g, const uint32_t* step_ptr, const int* abort, int64_t nmax,
                        long long* words3);
// convect_particles! + get_cell for the fused variable-weight step: slots
// [0, *hw_dev), dead slots skipped, destination counts into the species'
// counts for the next sort
void launch_convect_count(mz_domain* d, int s, const mz_grid1d* g, const mz_walls1d* w, double dt,
                          const uint32_t* step_ptr, const long long* hw_dev, const int* abort, double* surf);
void launch_step(mz_domain* d, const mz_step_plan* plan, int64_t n_steps, mz_props* inst, mz_props* avg);
void autotune_step(mz_domain* d, const mz_step_plan* plan, int64_t trial_steps, int32_t* lanes_out, int32_t* big_out);
void launch_fill_i32(mz_ctx* c, int32_t* p, int64_t n, int32_t v);
void reserve_species(mz_domain* d, int s, int64_t cap);
void launch_key_from_cell(mz_domain* d, int s);
void free_slab_scratch(mz_domain* d);
void launch_avg(mz_ctx* c, double* avg, const double* inst, int64_t n, double inv);

// Lanes per cell in the NTC kernels.  A conflict-free batch of a cell with n
// particles holds about sqrt(pi n / 8) candidates (12 at n = 400), and one warp
// instruction serves all of a warp's groups, so 8-lane groups (four cells per
// warp) use the FP64 pipe best; with few cells, wider groups shorten the
// sequential chain of each cell instead.
// cells per tile of the two-pass cell scan (sort.cu)
#define MZ_SCAN_TILE 2048
inline int64_t scan_tiles(int64_t cells) { return (cells + MZ_SCAN_TILE - 1) / MZ_SCAN_TILE; }

inline int ntc_group_width(int64_t cells)
{
    return cells >= 4096 ? 8 : (cells >= 1024 ? 16 : 32);
}

#define MZ_LAUNCH(ctx, name, kernel, grid, block, smem, ...)                                           \
    do {                                                                                               \
        cudaEvent_t _ev0 = nullptr;                                                                    \
        int _slot = (ctx)->timer_begin(name, &_ev0);                                                   \
        kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                               \
        MZ_CK(cudaGetLastError());                                                                     \
        (ctx)->launches++;                                                                             \
        (ctx)->timer_end(_slot, _ev0);                                                                 \
    } while (0)
