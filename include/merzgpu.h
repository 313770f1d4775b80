/*
 * merzgpu -- GB300 (sm_103a) implementation of Merzbild.jl's per-step DSMC hot
 * path behind a plain C ABI.
 *
 * Conventions
 *   - Every function returns an int status: MZ_OK (0) or an MZ_E_* code.
 *     mz_last_error() returns the message of the last failure on a context.
 *   - Indices are 0-based.  Merzbild.jl is 1-based; a Julia binding adds or
 *     subtracts 1 at the boundary (cells, slots, indexer fields).
 *   - Host pointers passed in are only read during the call (copied); output
 *     pointers are written before the call returns.
 *   - A domain is bound to one context (one device, one stream).  Calls on a
 *     domain are enqueued on that stream and may return before the device has
 *     finished; functions that return data to the host synchronize.  Handles
 *     are not thread-safe: use one host thread per context.
 *   - Array layouts of property outputs follow Merzbild.jl's Julia
 *     column-major arrays so a binding can pass its arrays straight through:
 *     np/n/T are (n_cells, n_species), v is (3, n_cells, n_species), moments is
 *     (n_moments, n_cells, n_species).
 *   - Random numbers are counter-based (Philox4x32-10); every call that draws
 *     takes an explicit `step` and draws from streams keyed on
 *     (seed, step, cell, particle/candidate), so results do not depend on
 *     launch shape, batching, or the order of cells.
 */
#ifndef MERZGPU_H
#define MERZGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MZ_ABI_VERSION 3
#define MZ_MAX_SPECIES 4

enum {
    MZ_OK = 0,
    MZ_E_ARG = 1,       /* invalid argument */
    MZ_E_CUDA = 2,      /* CUDA runtime error */
    MZ_E_CAPACITY = 3,  /* particle storage full (grow with mz_domain_reserve) */
    MZ_E_TIMEOUT = 4,   /* a bounded device wait gave up */
    MZ_E_STATE = 5,     /* device status word reported a failed invariant */
    MZ_E_NOMEM = 6      /* device allocation failed */
};

/* flags */
#define MZ_NTC_EQUAL_WEIGHT 1        /* ntc_equal_weight! semantics (no splitting) */
#define MZ_CONVECT_COMPUTE_CELL 1    /* convect_particles_and_compute_cell! */
#define MZ_PROPS_ALL 0               /* compute_props!: group1 and group2 */
#define MZ_PROPS_MOMENTS 1           /* compute_props_with_total_moments! */
#define MZ_PROPS_SORTED 2            /* compute_props_sorted!: group1 only */

typedef struct mz_ctx_s mz_ctx;
typedef struct mz_domain_s mz_domain;
typedef struct mz_props_s mz_props;
typedef struct mz_surf_props_s mz_surf_props;

/* Interaction (collision_utils.jl:73-82) */
typedef struct {
    double m_r, mu1, mu2, vhs_d, vhs_o, vhs_Tref, vhs_muref, vhs_factor;
} mz_interaction;

/* ParticleIndexer (particles.jl:56-66), 0-based slots, empty group: start 0, end -1 */
typedef struct {
    int64_t n_local, start1, end1, n_group1, start2, end2, n_group2;
} mz_particle_indexer;

/* CollisionFactors (collision_ntc.jl:18-25) */
typedef struct {
    int64_t n1, n2;
    double sigma_g_w_max;
    int64_t n_coll, n_coll_performed, n_eq_w_coll_performed;
} mz_collision_factors;

/* Grid1DUniform (grid_uniform1D.jl:49-86) */
typedef struct {
    double L;
    int64_t n_cells;
    double dx, inv_dx, min_x, max_x;
} mz_grid1d;

/* MaxwellWalls1D (boundary_conditions.jl:29-53); wall 0 = left, 1 = right */
typedef struct {
    double T[2];
    double v[2][3];
    double accommodation[2];
    double reflection_v_sq[2][MZ_MAX_SPECIES]; /* 2 k_B T_wall / m_species */
} mz_walls1d;

/* OctreeN2Merge options (merging_octree_N2.jl:235-246) */
typedef struct {
    int32_t split;              /* 1 = OctreeBinMidSplit (the only split implemented) */
    int32_t init_bin_bounds;    /* 1 = MinMaxVel, 2 = MinMaxVelSym, 3 = C */
    int32_t bin_bounds_compute; /* 1 = Inherit, 2 = Recompute */
    int32_t max_Nbins;
    int32_t max_depth;
} mz_octree_params;

typedef struct {
    unsigned long long candidates, accepted, splits, merges, wall_hits;
} mz_counters;

/* Fused multi-step driver: one step = ntc (every species pair, reference
 * order) -> convect + cell (1D) -> counting sort -> compute_props_sorted! /
 * compute_props! -> avg_props!.  Mirrors the time loops of
 * simulations/1D/couette_benchmarking.jl:58-85 and README.md:91-106. */
typedef struct {
    int32_t dims;         /* 0: 0D cells (no convection, no sort); 1: 1D grid */
    int32_t collide;      /* 1: run NTC each step */
    int32_t equal_weight; /* 1: ntc_equal_weight!; 0: ntc! with weight splitting and octree merging
                             (merge_* below); one species runs device-resident and graph-replayed,
                             a mixture runs the standalone entry points step by step */
    int32_t props;        /* 1: compute props at the end of every step */
    int64_t avg_start;    /* 1-based step of this call from which props are averaged; <= 0: never */
    int64_t n_avg;        /* avg_props! denominator */
    double dt;
    double dw_tol;
    uint64_t step0;       /* RNG step index of the first step */
    int32_t use_graph;    /* capture the step in a CUDA graph and replay it */
    int32_t big_cell;     /* 0-D: cells of at least this many particles collide one block per cell
                             (0: 2,048; < 0: never); results do not depend on it */
    mz_grid1d grid;
    mz_walls1d walls;
    int32_t launches;     /* 1-D: 1 (one fused launch), 2 (sort + gather + props, then NTC + convection
                             in a second launch) or 3 (one launch in which some warps of every block sort,
                             gather and compute props cell by cell while the others collide and convect
                             the cells already gathered); 0: the autotuner's choice, else 1.  Results do
                             not depend on it */
    int64_t hit_queue_capacity; /* 1-D: entries of the queue of particles that reach a wall (0: a
                                   sixteenth of the particles, at least 4,096); particles beyond it are
                                   reflected inside the step kernel.  Results do not depend on it */
    /* equal_weight = 0: the variable-weight loop of
     * simulations/1D/couette_varweight_octree.jl:85-135 (dims = 1) and of the
     * 0-D variable-weight tests -- per cell ntc! with splitting, then
     * merge_octree_N2_based! of the cells holding more than merge_threshold
     * particles down to merge_target (1-D: positions clamped to the grid) --
     * before convection (1-D), sort and props.  merge_threshold <= 0: no
     * merging.  A step that would overflow the storage is abandoned before it
     * changes a particle; the call grows the storage (mz_domain_reserve) and
     * resumes, so results equal an uninterrupted run. */
    int64_t merge_threshold;
    int64_t merge_target;
    mz_octree_params octree;
    int32_t split_lanes;  /* equal_weight = 0: lanes per cell of the splitting NTC, 8, 16 or 32; 0:
                             the autotuner's choice, else 32.  Results do not depend on it */
} mz_step_plan;

/* ---------------------------------------------------------------- context */
int mz_version(void);
int mz_ctx_create(int device, mz_ctx** out);
int mz_ctx_destroy(mz_ctx* ctx);
int mz_ctx_synchronize(mz_ctx* ctx);
int mz_last_error(const mz_ctx* ctx, char* buf, size_t len);
/* the context's cudaStream_t, for callers that record their own events */
int mz_ctx_stream(mz_ctx* ctx, void** stream);
/* event timing on the context stream */
int mz_timer_start(mz_ctx* ctx);
int mz_timer_stop(mz_ctx* ctx, double* ms);
/* write a scratch buffer larger than L2 (cache flush between timed runs) */
int mz_ctx_flush_l2(mz_ctx* ctx);
/* per-kernel CUDA-event timing of the library's own launches (0 = off) */
int mz_ctx_set_kernel_timing(mz_ctx* ctx, int enable);
/* name, total ms and launch count of timed kernel k (k < *n_kernels) */
int mz_kernel_timing(mz_ctx* ctx, int k, char* name, size_t len, double* total_ms, int64_t* launches,
                     int* n_kernels);
/* number of library kernels launched since context creation */
int mz_launch_count(mz_ctx* ctx, int64_t* launches);

/* ---------------------------------------------------------------- domain */
/* ParticleIndexerArray(n_cells, n_species) + ParticleVector(capacity[s]) per
 * species + the CollisionFactors array of all pairs and cells. */
int mz_domain_create(mz_ctx* ctx, int64_t n_cells, int32_t n_species, const int64_t* capacity, mz_domain** out);
int mz_domain_destroy(mz_domain* dom);
/* grow a species' storage (Base.resize!, particles.jl:269-298) */
int mz_domain_reserve(mz_domain* dom, int32_t species, int64_t capacity);
int mz_domain_info(mz_domain* dom, int32_t species, int64_t* capacity, int64_t* n_total, int64_t* high_water);
/* species masses (load_species_data, particles.jl:580-591) */
int mz_set_species(mz_domain* dom, const double* mass);
/* interactions [s1 + n_species * s2] (load_interaction_data, collision_utils.jl:159-202) */
int mz_set_interactions(mz_domain* dom, const mz_interaction* inter);
/* cell volumes (Grid1DUniform cells V / 0-D V); NULL resets to 1.0 */
int mz_set_cell_volumes(mz_domain* dom, const double* V);
int mz_set_seed(mz_domain* dom, uint64_t seed);
/* per-cell RNG keys for independent instances sharing one domain: seed,
 * stream id and step offset per cell; NULL arrays reset to the domain defaults */
int mz_set_cell_rng(mz_domain* dom, const uint64_t* seed, const uint32_t* rid, const uint32_t* step_offset);

/* ---------------------------------------------------------------- particles */
/* Load n particles of one species (w[n], v[n][3], x[n][3], cell[n] 0-based).
 * The layout is sorted by cell (stable in the given order), every cell's
 * particles in group 1: the state sample_particles_equal_weight! +
 * sort_particles! leave (distributions_and_sampling.jl:477-509). */
int mz_upload_particles(mz_domain* dom, int32_t species, int64_t n, const double* w, const double* v, const double* x,
                        const int32_t* cell);
/* Load raw slots plus an explicit indexer (n_cells entries, 0-based slots);
 * slots no indexer entry covers are dead.  Reproduces hand-built
 * ParticleIndexerArray states of the reference tests. */
int mz_upload_particles_indexed(mz_domain* dom, int32_t species, int64_t n_slots, const double* w, const double* v,
                                const double* x, const mz_particle_indexer* indexer);
/* Particles in logical order (cells ascending, each cell's group1 then
 * group2: pv[i] over the indexer); *n_out = n_total.  cell may be NULL. */
int mz_download_particles(mz_domain* dom, int32_t species, int64_t max_n, double* w, double* v, double* x,
                          int32_t* cell, int64_t* n_out);
int mz_get_indexer(mz_domain* dom, int32_t species, mz_particle_indexer* out, int64_t* n_total);

/* ---------------------------------------------------------------- collisions */
int mz_set_collision_factors(mz_domain* dom, int32_t s1, int32_t s2, const double* sigma_g_w_max);
int mz_get_collision_factors(mz_domain* dom, int32_t s1, int32_t s2, mz_collision_factors* out);
/* ntc! / ntc_equal_weight! for cells [cell_begin, cell_end) of pair (s1, s2):
 * single species when s1 == s2 (collision_ntc.jl:338-380, :479-521), two
 * species otherwise (collision_ntc.jl:412-453, :554-595).  Cell volumes from
 * mz_set_cell_volumes.  Split particles (dw_tol, collision_ntc.jl:223-270) go
 * to the cell's group 2. */
int mz_ntc(mz_domain* dom, int32_t s1, int32_t s2, double dt, int64_t cell_begin, int64_t cell_end, uint64_t step,
           int32_t flags, double dw_tol);

/* swpm!(rng, collision_factors_swpm, collision_data, interaction, particles,
 * pia, cell, species, G, dt, V) (collision_swpm.jl:201-288) for cells
 * [cell_begin, cell_end) of one species, G >= 0.  The pair (species,
 * species)'s collision factors hold CollisionFactorsSWPM
 * (collision_swpm.jl:18-24): set (sigma g)_max with mz_set_collision_factors
 * (create_collision_factors_swpm_array: estimate_sigma_g_w_max with Fnum = 1),
 * read sigma_g_max, n_coll and n_coll_performed back with
 * mz_get_collision_factors (field sigma_g_w_max).  Every accepted collision
 * appends two particles to the cell's group 2.  Draws come from the NTC
 * streams of the pair. */
int mz_swpm(mz_domain* dom, int32_t species, double G, double dt, int64_t cell_begin, int64_t cell_end,
            uint64_t step);

/* ---------------------------------------------------------------- properties */
/* PhysProps(n_cells, n_species, moments_list; ndens_not_Np, Tref) (physical_props.jl:24-58) */
int mz_props_create(mz_domain* dom, int32_t n_moments, const int32_t* moment_powers, double Tref, int32_t ndens_not_Np,
                    mz_props** out);
int mz_props_destroy(mz_props* p);
/* compute_props! / compute_props_with_total_moments! / compute_props_sorted! (MZ_PROPS_*) */
int mz_compute_props(mz_domain* dom, mz_props* p, int32_t mode);
/* avg_props! (physical_props.jl:281-299) */
int mz_avg_props(mz_props* avg, const mz_props* inst, double n_avg_timesteps);
/* clear_props! (physical_props.jl:256-262) */
int mz_clear_props(mz_props* p);
/* copy to host; any pointer may be NULL */
int mz_props_download(mz_props* p, double* lpa, double* np, double* n, double* v, double* T, double* moments);
/* Read a property set back without stopping the device: np, n, v and T (the
 * layouts of mz_props_download, back to back: 6 n_cells n_species doubles)
 * are copied into one of two device snapshot buffers (slot 0 or 1) after the
 * work already enqueued, and from there to host memory `dst` on a side
 * stream while later work runs.  dst must stay valid until
 * mz_props_snapshot_wait(p, slot) returns; page-locked memory (mz_host_alloc)
 * makes the copy asynchronous.  A slot is refilled only after its previous
 * host copy has finished.  No counterpart in the reference (its loops read
 * phys_props on the host). */
int mz_props_snapshot(mz_props* p, int32_t slot, double* dst);
int mz_props_snapshot_wait(mz_props* p, int32_t slot);
/* page-locked host memory for asynchronous copies */
int mz_host_alloc(mz_ctx* ctx, size_t bytes, void** out);
int mz_host_free(void* ptr);

/* ---------------------------------------------------------------- convection */
/* convect_particles! (convection_1D.jl:130-157) or, with
 * MZ_CONVECT_COMPUTE_CELL, convect_particles_and_compute_cell! (:225-255).
 * grid: the domain's grid or, without MZ_CONVECT_COMPUTE_CELL, the global
 * grid that a slab domain is part of (mz_slab_extract) */
int mz_convect_1d(mz_domain* dom, int32_t species, const mz_grid1d* grid, const mz_walls1d* walls, double dt,
                  uint64_t step, int32_t flags);

/* Surface properties of the two walls of a 1-D grid: SurfProps(pia, grid)
 * (surface_props.jl:22-67; element 1 = left wall, normal +x, element 2 =
 * right wall, normal -x, unit areas).  Downloads use the reference's layouts:
 * np, flux_incident, flux_reflected, normal_pressure, kinetic_energy_flux are
 * (2, n_species), force and shear_pressure (3, 2, n_species), column-major.
 * Sums are accumulated with atomic additions: equal to the sequential sums up
 * to round-off, not bit for bit. */
int mz_surf_props_create(mz_domain* dom, mz_surf_props** out);
int mz_surf_props_destroy(mz_surf_props* surf);
/* clear_props!(surf_props) (surface_props.jl:176-196) */
int mz_surf_props_clear(mz_surf_props* surf);
/* avg_props!(surf_props_avg, surf_props, n_avg_timesteps) (surface_props.jl:205-226) */
int mz_surf_avg_props(mz_surf_props* avg, const mz_surf_props* inst, double n_avg_timesteps);
int mz_surf_props_download(mz_surf_props* surf, double* np, double* flux_incident, double* flux_reflected,
                           double* force, double* normal_pressure, double* shear_pressure, double* kinetic_energy_flux);
/* convect_particles!(rng, grid, boundaries, particles, pia, species,
 * species_data, surf_props, dt) (convection_1D.jl:176-206): this species'
 * entries are cleared, every wall hit adds its incident and reflected
 * contributions, and the sums are scaled by mass / dt / area
 * (surface_props_scale!).  (The reference clears every species' entries.) */
int mz_convect_1d_surf(mz_domain* dom, int32_t species, const mz_grid1d* grid, const mz_walls1d* walls, double dt,
                       uint64_t step, int32_t flags, mz_surf_props* surf);
/* Attach surface sets to the fused 1-D step: every step clears inst,
 * samples the walls during convection, scales, and (avg != NULL) adds inst /
 * plan->n_avg to avg from plan->avg_start on, like avg_props!.  NULL detaches.
 * No counterpart in the reference (its time loops call the functions above). */
int mz_step_set_surface(mz_domain* dom, mz_surf_props* inst, mz_surf_props* avg);

/* ---------------------------------------------------------------- netCDF output */
/* Output files of cell properties (NCDataHolder, io.jl:116-243) and surface
 * properties (NCDataHolderSurf, io.jl:430-547): the reference's dimensions,
 * variables (names, Float64 / Int32 types, dimension order) and skip lists, in
 * the netCDF classic 64-bit-offset container (the reference writes netCDF-4,
 * which needs HDF5).  species_names is a char variable (n_species,
 * species_name_length); a cell-property file without moments has no
 * n_moments dimension and no moment variables (classic netCDF has no
 * fixed dimension of length 0).
 * Writes from device sets (mz_nc_props_write, mz_nc_surf_write) are enqueued
 * on the context's stream after the work already there: the record is packed
 * on the device, copied to pinned memory on a side stream and written to the
 * file by the file's writer thread, so the caller does not wait for the disk.
 * The *_host forms take the reference's host arrays (column-major layouts of
 * mz_props_download / mz_surf_props_download).  ctx may be NULL for a file
 * written only from host arrays.  Handles are not thread-safe. */
typedef struct mz_nc_file_s mz_nc_file;
enum { MZ_NC_ATTR_TEXT = 0, MZ_NC_ATTR_INT = 1, MZ_NC_ATTR_DOUBLE = 2 };
/* one global attribute (NCDataHolder's global_attributes): count chars,
 * int32 values or doubles at `values` */
typedef struct {
    const char* name;
    int32_t type;
    int32_t count;
    const void* values;
} mz_nc_attribute;
/* NCDataHolder(nc_filename, names_skip_list, species_data, phys_props;
 * global_attributes) (io.jl:143-224); skip names as IOSkipList (io.jl:19-80):
 * length_particle_array, moments, np / nparticles, ndens, v, T.  Adds the
 * "COMMENT ndens" attribute.  The first n_names of the n_species entries of
 * species_names are set (the reference's putvar of species_data's names). */
int mz_nc_props_create(const char* path, const char* const* skip, int32_t n_skip, const char* const* species_names,
                       int32_t n_names, int32_t n_species, int32_t n_cells, int32_t n_moments, const int32_t* moment_powers,
                       int32_t ndens_not_Np, const mz_nc_attribute* gatts, int32_t n_gatts, mz_ctx* ctx,
                       mz_nc_file** out);
/* NCDataHolderSurf(nc_filename, names_skip_list, species_data, surf_props;
 * global_attributes) (io.jl:457-527); skip names as IOSkipListSurf
 * (io.jl:334-418): np / nparticles, fluxes, force, normal_pressure,
 * shear_pressure, kinetic_energy_flux. */
int mz_nc_surf_create(const char* path, const char* const* skip, int32_t n_skip, const char* const* species_names,
                      int32_t n_names, int32_t n_species, int32_t n_elements, const mz_nc_attribute* gatts, int32_t n_gatts,
                      mz_ctx* ctx, mz_nc_file** out);
/* write_netcdf(ds, phys_props, timestep; sync_freq) (io.jl:274-317): one
 * record; MZ_E_ARG if the set's ndens_not_Np differs from the file's (the
 * reference's ErrorException); sync_freq > 0 syncs the file to disk after
 * every sync_freq-th record. */
int mz_nc_props_write(mz_nc_file* f, const mz_props* p, double timestep, int32_t sync_freq);
int mz_nc_props_write_host(mz_nc_file* f, const double* lpa, const double* np, const double* ndens, const double* v,
                           const double* T, const double* moments, int32_t ndens_not_Np, double timestep,
                           int32_t sync_freq);
/* write_netcdf(ds, surf_props, timestep; sync_freq) (io.jl:566-603) */
int mz_nc_surf_write(mz_nc_file* f, const mz_surf_props* surf, double timestep, int32_t sync_freq);
int mz_nc_surf_write_host(mz_nc_file* f, const double* np, const double* flux_incident, const double* flux_reflected,
                          const double* force, const double* normal_pressure, const double* shear_pressure,
                          const double* kinetic_energy_flux, double timestep, int32_t sync_freq);
/* wait until every enqueued record is in the file; reports a failed write */
int mz_nc_flush(mz_nc_file* f);
/* records enqueued so far */
int mz_nc_records(const mz_nc_file* f, int64_t* n);
/* close_netcdf(ds) (io.jl:251-253): writes what is enqueued and closes */
int mz_nc_close(mz_nc_file* f);
int mz_nc_last_error(const mz_nc_file* f, char* buf, size_t len);

/* ---------------------------------------------------------------- sorting */
/* sort_particles!(gridsort, grid, ...) when grid != NULL (cells from x,
 * grid_sorting.jl:58-113), sort_particles!(gridsort, ...) with the cells
 * stored by convect_particles_and_compute_cell! otherwise (:128-182).
 * out_index (optional, n_total entries): for every sorted slot, the logical
 * position (0-based) it held before the sort -- the permutation the
 * reference writes into ParticleVector.index. */
int mz_sort(mz_domain* dom, int32_t species, const mz_grid1d* grid, int64_t* out_index);
/* squash_pia! (particles.jl:622-701): close the gaps left by deletions; each
 * cell's logical order is kept and every cell ends up in group 1 */
int mz_squash(mz_domain* dom, int32_t species);

/* ---------------------------------------------------------------- merging */
/* merge_octree_N2_based! (merging_octree_N2.jl:1060-1094) for every cell in
 * [cell_begin, cell_end) whose particle count exceeds `threshold`
 * (threshold < 0: every non-empty cell), batched in one launch.  grid != NULL
 * selects the 1-D variant that clamps new positions (:830-933).
 * *n_merged (optional) receives the number of merged cells. */
int mz_merge_octree_n2(mz_domain* dom, int32_t species, int64_t cell_begin, int64_t cell_end, int64_t threshold,
                       int64_t target_np, const mz_octree_params* params, const mz_grid1d* grid, uint64_t step,
                       int64_t* n_merged);

/* ---------------------------------------------------------------- sampling */
/* sample_particles_equal_weight! for a set of cells at once: counts[c]
 * particles in cell c (appended to the cell, which must be empty), velocities
 * Maxwellian with per-axis temperatures T3[c][3] (T3 NULL: T3_all) or BKW
 * (distribution 1, T3[c][0] as T), weights Fnum[c] * 10^(span * (2U - 1))
 * (span 0: equal weight), positions uniform in box6[c] = {xlo, xhi, ylo,
 * yhi, zlo, zhi} (NULL: unit cube), velocity offsets (the keywords vx0, vy0,
 * vz0) v0[c][3] or, with v0 NULL, v0_all[3] for every cell (both NULL: none).
 * (distributions_and_sampling.jl:432-509, 195-213, grid_uniform1D.jl:117-219) */
int mz_sample_cells(mz_domain* dom, int32_t species, const int64_t* counts, const double* T3, const double* T3_all,
                    const double* Fnum, double log10_weight_span, const double* box6, int32_t distribution,
                    uint64_t step, const double* v0, const double* v0_all);
/* sample_particles_equal_weight!(rng, grid, ..., ndens::Float64, T, Fnum; vx0, vy0, vz0)
 * (grid_uniform1D.jl:198-219); v0 = {vx0, vy0, vz0} or NULL */
int mz_sample_grid_ndens(mz_domain* dom, int32_t species, const mz_grid1d* grid, double ndens, double T, double Fnum,
                         uint64_t step, const double* v0);

/* ---------------------------------------------------------------- fused step */
/* n_steps steps of the fused pipeline; inst receives the props of the last
 * step, avg accumulates avg_props! from plan->avg_start (either may be NULL) */
int mz_step(mz_domain* dom, const mz_step_plan* plan, int64_t n_steps, mz_props* inst, mz_props* avg);

/* ---------------------------------------------------------------- serving */
/* No counterpart in the reference (its drivers run one simulation per
 * process).  A continuous-batching server of independent 0-D solves -- the
 * README's relaxation problem (README.md:91-106) as a request: particles of
 * each species sampled Maxwellian at their temperature in a cell of volume V,
 * then n_steps of ntc! for every species pair and compute_props!.  Each
 * request occupies one cell of a server domain while it runs; requests are
 * admitted first come first served while a cell and the per-species particle
 * budget (capacity) are free, running requests advance together in fused
 * steps, and a request's result depends only on the request (its seed), not
 * on the requests beside it or its cell.  Requests of at least 4,096
 * particles (mz_server_set_lane_split) run in a second lane -- a domain of
 * its own on a stream of its own -- while the smaller ones step on another
 * stream meanwhile, several of their steps per step of the large ones. */
typedef struct mz_server_s mz_server;

enum { MZ_REQ_QUEUED = 0, MZ_REQ_RUNNING = 1, MZ_REQ_DONE = 2 };

typedef struct {
    int64_t count[MZ_MAX_SPECIES]; /* particles per species (0: species absent) */
    double T[MZ_MAX_SPECIES];      /* initial temperature per species, K */
    double Fnum;                   /* particle weight */
    double V;                      /* cell volume */
    int64_t n_steps;               /* time steps, >= 1 */
    uint64_t seed;                 /* key of all of the request's random streams */
} mz_request;

typedef struct {
    int64_t id;
    int32_t state;       /* MZ_REQ_* */
    int32_t reserved;
    int64_t steps_done;
    int64_t np[MZ_MAX_SPECIES];          /* after the last step */
    double n[MZ_MAX_SPECIES];
    double v[MZ_MAX_SPECIES][3];
    double T[MZ_MAX_SPECIES];
} mz_request_result;

/* a server for up to max_requests concurrent requests of n_species species
 * (masses, interactions [s1 + n_species * s2] as mz_set_interactions), time
 * step dt; each of the two lanes holds up to max_requests requests and
 * capacity[s] particles of each species in HBM.  capacity[s] = 0 (any
 * species) admits by free device memory instead: a lane's storage grows when
 * an admission needs it and cudaMemGetInfo's free bytes, less the headroom
 * (mz_server_set_hbm_headroom, 2 GiB by default), hold the larger storage
 * (144 bytes per particle); a request that does not fit waits in its lane's
 * queue, and only a request larger than the whole device memory less the
 * headroom is refused at submission. */
int mz_server_create(mz_ctx* ctx, int32_t n_species, const double* mass, const mz_interaction* inter, double dt,
                     int64_t max_requests, const int64_t* capacity, mz_server** out);
int mz_server_destroy(mz_server* server);
/* queue a request; *id identifies it */
int mz_server_submit(mz_server* server, const mz_request* request, int64_t* id);
/* admit what fits, advance every running request by one step, retire the
 * finished ones; counts after the step */
int mz_server_step(mz_server* server, int64_t* n_running, int64_t* n_queued, int64_t* n_retired);
/* The same for up to max_steps steps in one call.  The lane of large
 * requests runs k steps, k = the fewest steps any of its running requests
 * still needs (at most max_steps), so no request steps past its end; while
 * they run, the lane of small requests runs such batches of steps one after
 * another, retiring and admitting between them.  *n_steps receives the
 * larger of the two lanes' step counts.  Results are those of single steps. */
int mz_server_step_many(mz_server* server, int64_t max_steps, int64_t* n_steps, int64_t* n_running,
                        int64_t* n_queued, int64_t* n_retired);
/* state of a request and, once done, its final properties */
int mz_server_result(mz_server* server, int64_t id, mz_request_result* out);
/* ids of the requests the last mz_server_step(_many) call retired (*n of them; up to
 * max_ids written) */
int mz_server_retired(mz_server* server, int64_t max_ids, int64_t* ids, int64_t* n);
/* steps run (by the lane that ran more) and particle-steps done so far */
int mz_server_info(mz_server* server, int64_t* steps_run, int64_t* particle_steps);
/* requests of at least `particles` particles (all species together) run in
 * the lane of large requests; 0 puts all requests in one lane.  Applies to
 * requests submitted afterwards.  Results do not depend on the lane. */
int mz_server_set_lane_split(mz_server* server, int64_t particles);
/* device memory admission by free memory keeps free (capacity 0 at creation) */
int mz_server_set_hbm_headroom(mz_server* server, int64_t bytes);

/* Choose the fused step's mapping by timing it: every combination of lanes
 * per cell in the warp-group NTC (8, 16, 32) and, for 0-D plans, of the
 * block-per-cell threshold (512, 2,048, 8,192 particles, never) or, for 1-D
 * plans, of the plan's launches 1, 2 and 3 runs trial_steps real steps of `plan` twice, in
 * two rounds of opposite order whose times add up (starting at
 * plan->step0; the state advances by
 * 24 * trial_steps steps for 0-D plans and 18 * trial_steps for 1-D, and
 * every mapping gives the same results); the fastest is kept for later
 * mz_step calls whose plan leaves big_cell at 0.  *big_cell_out receives the
 * threshold (0-D) or, for 1-D, the launches value minus one (0 fused, 1 two
 * launches, 2 gathering and physics warps side by side).  A variable-weight plan
 * (equal_weight = 0) tries only the lanes per cell of its splitting NTC (8,
 * 16, 32; 6 * trial_steps steps, without a graph), compares the splitting
 * NTC's own launch times (the lanes change nothing else), and *big_cell_out
 * receives 0.
 * No counterpart in the reference. */
int mz_step_autotune(mz_domain* dom, const mz_step_plan* plan, int64_t trial_steps, int32_t* lanes, int32_t* big_cell);

/* ---------------------------------------------------------------- counters */
int mz_get_counters(mz_domain* dom, mz_counters* out, int32_t reset);

/* ---------------------------------------------------------------- diagnostics */
/* No counterpart in the reference.  Evaluates, on the device, the sine and
 * cosine the collision kernels use for the scattering angle phi = 2 pi rand():
 * s[i], c[i] = sin, cos of 2 pi m[i] 2^-52 for 52-bit integers m[i] (the
 * uniform draw's mantissa).  Host arrays of n elements; for accuracy tests. */
int mz_sincos_2pi(mz_ctx* ctx, int64_t n, const uint64_t* m, double* s, double* c);

/* ---------------------------------------------------------------- slabs */
/* One 1-D grid over several GPUs, one process each (exchange_particles! and
 * sort_particles_after_exchange!, parallel.jl:281-532, move particles
 * between the cell chunks of a multithreaded run).  A rank's domain holds
 * the cells [c0, c0 + n_cells) of the global grid `grid` (give them the
 * global cell ids with mz_set_cell_rng, so every stream is the one a single
 * domain would draw), convects on the global grid and walls
 * (mz_convect_1d without MZ_CONVECT_COMPUTE_CELL), then:
 *   mz_slab_extract : frees the particles now outside the slab and stages
 *                     them, *n_left for the left neighbour and *n_right for
 *                     the right one, in slot order;
 *   mz_slab_fetch   : copies them to the host, 7 doubles per particle
 *                     (w, vx, vy, vz, x, y, z);
 *   mz_slab_insert  : after the caller's exchange with the neighbours,
 *                     rebuilds the storage as [from the left | own | from the
 *                     right] and sorts it by cell.
 * Every cell's particles end in the order a single domain over the whole
 * grid gives them, so a sharded equal-weight run equals the single-domain
 * run bit for bit.  A particle that crossed a whole neighbour's slab in one
 * step is clamped into the slab and reported (MZ_E_STATE). */
int mz_slab_extract(mz_domain* dom, int32_t species, const mz_grid1d* grid, int64_t c0, int64_t* n_left,
                    int64_t* n_right);
int mz_slab_fetch(mz_domain* dom, int32_t species, double* left, double* right);
int mz_slab_insert(mz_domain* dom, int32_t species, const mz_grid1d* grid, int64_t c0, const double* from_left,
                   int64_t n_left, const double* from_right, int64_t n_right);

/* ---------------------------------------------------------------- validators */
/* The reference's indexing checks (particles.jl:805-1025) on the device
 * layout of one species.  mode 0: check_pia_is_correct -- every cell's groups
 * have non-negative sizes and lie inside the slots in use, and the cells'
 * counts add up to n_total; *ok = 0 with *detail = the first bad cell
 * (1-based) or 0 for a wrong total.  mode 1: check_unique_index -- *ok = 0
 * when a slot is listed by more than one group (*detail = the largest count,
 * negated when free slots are listed as well) or a group lists a free slot
 * (*detail = -1).  mode 2: check_unique_buffer -- free slots are marked slot by
 * slot, so this always holds.  modes 3 and 4: count_disordered_particles with
 * and without per-cell offsets (use_offset), the count in *detail. */
int mz_check_indexing(mz_domain* dom, int32_t species, int32_t mode, int32_t* ok, int64_t* detail);
/* Write a species' indexer as given (a ParticleIndexerArray edited by hand,
 * as the reference's tests do): groups must lie inside the slots in use and
 * list no more particles than the storage holds; overlaps, free slots in
 * groups and an n_total that disagrees are accepted and left to the checks
 * above. */
int mz_set_indexer(mz_domain* dom, int32_t species, const mz_particle_indexer* indexer, int64_t n_total);

/* ---------------------------------------------------------------- no-allocation sort */
/* Largest n_cells mz_sort_keys_noalloc accepts.  Its scratch (per-cell counts
 * and cursors, 2 * 4 B per cell, 2 MiB) is a static device array that every
 * GPU loading the library holds until the process exits. */
#define MZ_NOALLOC_MAX_CELLS 262144

/* No counterpart in the reference.  The stable counting sort of n cell keys
 * (the permutation part of sort_particles!), for callers that must not
 * allocate device memory: a process whose device memory is owned by another
 * framework's caching allocator, or a loop that must not take the device-wide
 * synchronisation of cudaMalloc / cudaFree.  Everything is the caller's and in
 * device memory: d_keys[n] in [0, n_cells) (out-of-range keys are clamped and
 * reported as MZ_E_STATE), d_perm[n] receives for every sorted position the
 * index of the key that lands there (stable: equal keys keep their order),
 * d_cell_start[n_cells + 1] the exclusive prefix of the per-cell counts.
 * Runs on `stream` (a cudaStream_t, NULL = default stream) and, before
 * returning, waits for that stream (not for the whole device) to read the
 * out-of-range-key word.  Allocates nothing: the per-cell counters live in a
 * static device array shared by every call, cleared at the start of each
 * call; calls that overlap on the GPU race on it, so serialise them.  The
 * first call on a device -- and the first after that device's context was
 * reset -- looks up that array's device address (with the device current);
 * make that first call before any stream capture. */
int mz_sort_keys_noalloc(void* stream, const int32_t* d_keys, int64_t n, int32_t n_cells, int32_t* d_perm,
                         int32_t* d_cell_start);

#ifdef __cplusplus
}
#endif

#endif /* MERZGPU_H */
