"""
    MerzbildGPU

Julia binding of libmerzgpu.so (include/merzgpu.h): the per-step DSMC path of
Merzbild.jl (NTC collisions, 1-D convection, grid sorting, cell properties,
octree merging, sampling) on a GB300 GPU.

The module adds methods to Merzbild's own functions for device containers,
with the reference's positional arguments, so a time loop written against
Merzbild keeps its calls and swaps its containers:

    dp = DeviceParticles(DeviceContext(0), grid, species_data, interaction_data, capacity)
    particles, pia = device_particles(dp), DevicePIA(dp)
    collision_factors = create_collision_factors_array(pia, interaction_data, species_data, T, Fnum)
    rng = DeviceRNG(seed)
    for t in 1:n_timesteps
        for cell in 1:grid.n_cells
            ntc_equal_weight!(rng, collision_factors[1, 1, cell], collision_data, interaction_data,
                              particles[1], pia, cell, 1, Δt, grid.cells[cell].V)
        end
        convect_particles!(rng, grid, boundaries, particles[1], pia, 1, species_data, Δt)
        sort_particles!(DeviceGridSort(dp), grid, particles[1], pia, 1)
        compute_props_sorted!(particles, pia, species_data, phys_props)
    end

Its own forms take ranges of cells (one launch for many cells) and an
explicit step (`rng.step = t`), and `step!` runs whole fused steps replayed
from a CUDA graph.

Conventions at the boundary: the C ABI is 0-based (cells, slots); this
module takes and returns Merzbild's 1-based cells.  Random numbers come from
counter-based streams keyed on (seed, step, cell, particle), so `DeviceRNG`
carries a seed and the time-step index instead of a generator state.
"""
module MerzbildGPU

import Merzbild  # setup estimates (estimate_sigma_g_w_max) stay the reference's own
# the module's methods extend Merzbild's own functions, so a loop written
# against Merzbild dispatches to the device for device containers
import Merzbild: ntc!, ntc_equal_weight!, convect_particles!, convect_particles_and_compute_cell!, sort_particles!,
                 squash_pia!, compute_props!, compute_props_sorted!, compute_props_with_total_moments!,
                 avg_props!, clear_props!, merge_octree_N2_based!, sample_particles_equal_weight!, swpm!,
                 write_netcdf, close_netcdf, create_collision_factors_array, check_pia_is_correct,
                 check_unique_index, check_unique_buffer, count_disordered_particles

export DeviceContext, DeviceParticles, DeviceProps, DeviceRNG, DeviceGrid1D, DeviceWalls1D, DeviceOctree,
       upload!, download, ntc!, ntc_equal_weight!, convect_particles!, convect_particles_and_compute_cell!,
       sort_particles!, squash_pia!, compute_props!, compute_props_sorted!, compute_props_with_total_moments!,
       avg_props!, clear_props!, merge_octree_N2_based!, sample_particles_equal_weight!, step!, counters,
       DeviceSurfProps, set_step_surface!, DeviceNCDataHolder, DeviceNCDataHolderSurf, write_netcdf, close_netcdf,
       swpm!, create_collision_factors_swpm_array!, snapshot!, snapshot_wait, unpack_snapshot!, pinned_vector,
       free_pinned!, DeviceServer, submit!, server_step!, request_result, retired_requests, set_lane_split!,
       set_hbm_headroom!, DevicePIA, DeviceParticleVector, device_particles, DeviceCollisionFactors, DeviceGridSort,
       set_cell_volumes!, set_indexer!, check_pia_is_correct, check_unique_index, check_unique_buffer,
       count_disordered_particles, create_collision_factors_array

const libmz = joinpath(@__DIR__, "..", "merzgpu", "lib", "libmerzgpu.so")
const MZ_MAX_SPECIES = 4
const MZ_NTC_EQUAL_WEIGHT = Int32(1)
const MZ_CONVECT_COMPUTE_CELL = Int32(1)
const MZ_PROPS_ALL, MZ_PROPS_MOMENTS, MZ_PROPS_SORTED = Int32(0), Int32(1), Int32(2)

# ------------------------------------------------------------------ C structs
struct MzInteraction          # Interaction (collision_utils.jl:73-82)
    m_r::Float64; μ1::Float64; μ2::Float64; vhs_d::Float64; vhs_o::Float64
    vhs_Tref::Float64; vhs_muref::Float64; vhs_factor::Float64
end

struct MzParticleIndexer      # ParticleIndexer, 0-based slots
    n_local::Int64; start1::Int64; end1::Int64; n_group1::Int64
    start2::Int64; end2::Int64; n_group2::Int64
end

struct MzCollisionFactors
    n1::Int64; n2::Int64; sigma_g_w_max::Float64
    n_coll::Int64; n_coll_performed::Int64; n_eq_w_coll_performed::Int64
end

struct DeviceGrid1D           # Grid1DUniform (grid_uniform1D.jl:49-86)
    L::Float64; n_cells::Int64; dx::Float64; inv_dx::Float64; min_x::Float64; max_x::Float64
end
DeviceGrid1D(grid) = DeviceGrid1D(grid.L, grid.n_cells, grid.Δx, grid.inv_Δx, grid.min_x, grid.max_x)

struct DeviceWalls1D          # MaxwellWalls1D (boundary_conditions.jl:29-53), left then right
    T::NTuple{2,Float64}
    v::NTuple{6,Float64}
    accommodation::NTuple{2,Float64}
    reflection_v_sq::NTuple{2 * MZ_MAX_SPECIES,Float64}
end
function DeviceWalls1D(walls)
    ns = size(walls.reflection_velocities_sq, 2)   # (wall, species)
    vsq = ntuple(i -> begin
                     w, s = divrem(i - 1, MZ_MAX_SPECIES)
                     s < ns ? walls.reflection_velocities_sq[w + 1, s + 1] : 0.0
                 end, 2 * MZ_MAX_SPECIES)
    DeviceWalls1D((walls.boundaries[1].T, walls.boundaries[2].T),
                  (walls.boundaries[1].v..., walls.boundaries[2].v...),
                  (walls.boundaries[1].accommodation, walls.boundaries[2].accommodation), vsq)
end

struct DeviceOctree           # OctreeN2Merge options (merging_octree_N2.jl:235-246)
    split::Int32; init_bin_bounds::Int32; bin_bounds_compute::Int32; max_Nbins::Int32; max_depth::Int32
end
DeviceOctree(; init_bin_bounds=1, bin_bounds_compute=1, max_Nbins=4096, max_depth=10) =
    DeviceOctree(1, init_bin_bounds, bin_bounds_compute, max_Nbins, max_depth)

struct MzCounters
    candidates::UInt64; accepted::UInt64; splits::UInt64; merges::UInt64; wall_hits::UInt64
end

struct MzStepPlan
    dims::Int32; collide::Int32; equal_weight::Int32; props::Int32
    avg_start::Int64; n_avg::Int64; dt::Float64; dw_tol::Float64; step0::UInt64
    use_graph::Int32; big_cell::Int32
    grid::DeviceGrid1D; walls::DeviceWalls1D
    launches::Int32
    hit_queue_capacity::Int64
    merge_threshold::Int64; merge_target::Int64; octree::DeviceOctree
    split_lanes::Int32
end

# ------------------------------------------------------------------ handles
mutable struct DeviceContext
    ptr::Ptr{Cvoid}
    function DeviceContext(device::Integer=0)
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:mz_ctx_create, libmz), Cint, (Cint, Ref{Ptr{Cvoid}}), device, r), C_NULL)
        c = new(r[])
        finalizer(c -> ccall((:mz_ctx_destroy, libmz), Cint, (Ptr{Cvoid},), c.ptr), c)
        c
    end
end

mutable struct DeviceParticles
    ctx::DeviceContext
    ptr::Ptr{Cvoid}
    n_cells::Int
    n_species::Int
    V::Vector{Float64}   # host copy of the cell volumes on the device
end

"""
    DeviceParticles(ctx, n_cells, species_data, interactions, capacity; seed=1234)

Device counterpart of `particles::Vector{ParticleVector}`, `pia` and the
collision factors of all species pairs.
"""
function DeviceParticles(ctx::DeviceContext, n_cells, species_data, interactions, capacity; seed=1234)
    ns = length(species_data)
    cap = fill(Int64(capacity), ns)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:mz_domain_create, libmz), Cint, (Ptr{Cvoid}, Int64, Int32, Ptr{Int64}, Ref{Ptr{Cvoid}}),
                ctx.ptr, n_cells, ns, cap, r), ctx)
    dp = DeviceParticles(ctx, r[], n_cells, ns, ones(n_cells))
    finalizer(d -> ccall((:mz_domain_destroy, libmz), Cint, (Ptr{Cvoid},), d.ptr), dp)
    check(ccall((:mz_set_species, libmz), Cint, (Ptr{Cvoid}, Ptr{Float64}), dp.ptr, [s.mass for s in species_data]), ctx)
    tab = [MzInteraction(interactions[s1, s2].m_r, interactions[s1, s2].μ1, interactions[s1, s2].μ2,
                         interactions[s1, s2].vhs_d, interactions[s1, s2].vhs_o, interactions[s1, s2].vhs_Tref,
                         interactions[s1, s2].vhs_muref, interactions[s1, s2].vhs_factor) for s1 in 1:ns, s2 in 1:ns]
    check(ccall((:mz_set_interactions, libmz), Cint, (Ptr{Cvoid}, Ptr{MzInteraction}), dp.ptr, tab), ctx)
    check(ccall((:mz_set_seed, libmz), Cint, (Ptr{Cvoid}, UInt64), dp.ptr, seed), ctx)
    dp
end

mutable struct DeviceProps
    dp::DeviceParticles
    ptr::Ptr{Cvoid}
    n_moments::Int
    moment_powers::Vector{Int32}
    ndens_not_Np::Bool
end

"""
    DeviceProps(dp; moments_list=Int32[], Tref=300.0, ndens_not_Np=false)

Device counterpart of `PhysProps` (physical_props.jl:24-58); `fetch!` copies
into a `PhysProps`.
"""
function DeviceProps(dp::DeviceParticles; moments_list=Int32[], Tref=300.0, ndens_not_Np=false)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    m = Int32.(moments_list)
    check(ccall((:mz_props_create, libmz), Cint, (Ptr{Cvoid}, Int32, Ptr{Int32}, Float64, Int32, Ref{Ptr{Cvoid}}),
                dp.ptr, length(m), m, Tref, ndens_not_Np ? 1 : 0, r), dp.ctx)
    p = DeviceProps(dp, r[], length(m), m, ndens_not_Np)
    finalizer(q -> ccall((:mz_props_destroy, libmz), Cint, (Ptr{Cvoid},), q.ptr), p)
    p
end

"""
Seed and time-step index of the counter-based streams (replaces `rng`).

The functions with the reference's signatures (`ntc!(rng, collision_factors,
...)` etc.) advance `step` themselves: a call that comes back to a cell that
the same kind of call (and species pair) already drew for in the current
step starts the next step -- the reference's drivers visit every cell once per
step in increasing order.  The functions of this module's own forms take
`step` as it is.
"""
mutable struct DeviceRNG
    seed::UInt64
    step::UInt64
    seen::Dict{Tuple{Symbol,Int,Int},Int}  # (kind, species1, species2) => last cell drawn for in this step
end
DeviceRNG(seed::Integer) = DeviceRNG(UInt64(seed), UInt64(0), Dict{Tuple{Symbol,Int,Int},Int}())
DeviceRNG(seed::Integer, step::Integer) = DeviceRNG(UInt64(seed), UInt64(step), Dict{Tuple{Symbol,Int,Int},Int}())

function drop_in_step!(rng::DeviceRNG, kind::Symbol, species1::Integer, species2::Integer, cell::Integer)
    key = (kind, Int(species1), Int(species2))
    if rng.step == 0 || cell <= get(rng.seen, key, 0)
        rng.step += 1
        empty!(rng.seen)
    end
    rng.seen[key] = cell
    rng.step
end

function check(rc, ctx)
    rc == 0 && return nothing
    msg = ""
    cp = ctx isa DeviceContext ? ctx.ptr : ctx
    if cp != C_NULL
        buf = Vector{UInt8}(undef, 1024)
        ccall((:mz_last_error, libmz), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), cp, buf, length(buf))
        msg = unsafe_string(pointer(buf))
    end
    throw(ErrorException("merzgpu error $rc: $msg"))
end

cellrange(cell::Integer) = (Int64(cell - 1), Int64(cell))
cellrange(cells::Tuple) = (Int64(cells[1] - 1), Int64(cells[2]))

# ------------------------------------------------------------------ particles
"""Load particles of `species` (w, v as 3×n, x as 3×n, 1-based cells)."""
function upload!(dp::DeviceParticles, species, w::Vector{Float64}, v::Matrix{Float64}, x::Matrix{Float64},
                 cells::Vector{<:Integer})
    c0 = Int32.(cells .- 1)
    check(ccall((:mz_upload_particles, libmz), Cint,
                (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
                dp.ptr, species - 1, length(w), w, v, x, c0), dp.ctx)
end

"""Particles of `species` in logical order: (w, v 3×n, x 3×n, 1-based cells)."""
function download(dp::DeviceParticles, species)
    n = Ref{Int64}(0)
    check(ccall((:mz_get_indexer, libmz), Cint, (Ptr{Cvoid}, Int32, Ptr{MzParticleIndexer}, Ref{Int64}),
                dp.ptr, species - 1, C_NULL, n), dp.ctx)
    w = Vector{Float64}(undef, n[]); v = Matrix{Float64}(undef, 3, n[]); x = Matrix{Float64}(undef, 3, n[])
    cells = Vector{Int32}(undef, n[])
    check(ccall((:mz_download_particles, libmz), Cint,
                (Ptr{Cvoid}, Int32, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Ref{Int64}),
                dp.ptr, species - 1, n[], w, v, x, cells, n), dp.ctx)
    w, v, x, cells .+ 1
end

# ------------------------------------------------------------------ collisions
"""ntc! (collision_ntc.jl:338, :412) for one cell or a range (first, last) of cells."""
function ntc!(rng::DeviceRNG, dp::DeviceParticles, cell, species1, species2, Δt; dw_tol=1e-16)
    cb, ce = cellrange(cell)
    check(ccall((:mz_ntc, libmz), Cint, (Ptr{Cvoid}, Int32, Int32, Float64, Int64, Int64, UInt64, Int32, Float64),
                dp.ptr, species1 - 1, species2 - 1, Δt, cb, ce, rng.step, 0, dw_tol), dp.ctx)
end
ntc!(rng::DeviceRNG, dp::DeviceParticles, cell, species, Δt; dw_tol=1e-16) =
    ntc!(rng, dp, cell, species, species, Δt; dw_tol=dw_tol)

"""ntc_equal_weight! (collision_ntc.jl:479, :554)."""
function ntc_equal_weight!(rng::DeviceRNG, dp::DeviceParticles, cell, species1, species2, Δt)
    cb, ce = cellrange(cell)
    check(ccall((:mz_ntc, libmz), Cint, (Ptr{Cvoid}, Int32, Int32, Float64, Int64, Int64, UInt64, Int32, Float64),
                dp.ptr, species1 - 1, species2 - 1, Δt, cb, ce, rng.step, MZ_NTC_EQUAL_WEIGHT, 1e-16), dp.ctx)
end
ntc_equal_weight!(rng::DeviceRNG, dp::DeviceParticles, cell, species, Δt) =
    ntc_equal_weight!(rng, dp, cell, species, species, Δt)

"""
    swpm!(rng, dp, cell, species, G, Δt)

swpm! (collision_swpm.jl:201-288) for one cell or a range (first, last);
(σ g)_max per cell is the pair's collision factor
(`create_collision_factors_swpm_array!`).
"""
function swpm!(rng::DeviceRNG, dp::DeviceParticles, cell, species, G, Δt)
    cb, ce = cellrange(cell)
    check(ccall((:mz_swpm, libmz), Cint, (Ptr{Cvoid}, Int32, Float64, Float64, Int64, Int64, UInt64),
                dp.ptr, species - 1, G, Δt, cb, ce, rng.step), dp.ctx)
end

"""(σ g)_max of every species pair in every cell: estimate_sigma_g_w_max with
Fnum = 1 (create_collision_factors_swpm_array, collision_swpm.jl:118-149)."""
function create_collision_factors_swpm_array!(dp::DeviceParticles, interactions, species_data, T_list;
                                              mult_factor=1.0)
    for s2 in 1:dp.n_species, s1 in 1:dp.n_species
        v = Merzbild.estimate_sigma_g_w_max(interactions[s1, s2], species_data[s1], species_data[s2], T_list[s1],
                                            T_list[s2], 1.0; mult_factor=mult_factor)
        set_sigma_g_w_max!(dp, s1, s2, fill(v, dp.n_cells))
    end
end

"""Set (σ g w)_max of a species pair for every cell (create_collision_factors_array)."""
function set_sigma_g_w_max!(dp::DeviceParticles, species1, species2, values::Vector{Float64})
    check(ccall((:mz_set_collision_factors, libmz), Cint, (Ptr{Cvoid}, Int32, Int32, Ptr{Float64}),
                dp.ptr, species1 - 1, species2 - 1, values), dp.ctx)
end

function set_cell_volumes!(dp::DeviceParticles, V::Vector{Float64})
    check(ccall((:mz_set_cell_volumes, libmz), Cint, (Ptr{Cvoid}, Ptr{Float64}), dp.ptr, V), dp.ctx)
    dp.V .= V
end

# ------------------------------------------------------------------ convection and sorting
"""convect_particles! (convection_1D.jl:130-157)."""
convect_particles!(rng::DeviceRNG, grid::DeviceGrid1D, walls::DeviceWalls1D, dp::DeviceParticles, species, Δt) =
    check(ccall((:mz_convect_1d, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ref{DeviceGrid1D}, Ref{DeviceWalls1D}, Float64, UInt64, Int32),
                dp.ptr, species - 1, grid, walls, Δt, rng.step, 0), dp.ctx)

"""convect_particles_and_compute_cell! (convection_1D.jl:225-255)."""
convect_particles_and_compute_cell!(rng::DeviceRNG, grid::DeviceGrid1D, walls::DeviceWalls1D, dp::DeviceParticles,
                                    species, Δt) =
    check(ccall((:mz_convect_1d, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ref{DeviceGrid1D}, Ref{DeviceWalls1D}, Float64, UInt64, Int32),
                dp.ptr, species - 1, grid, walls, Δt, rng.step, MZ_CONVECT_COMPUTE_CELL), dp.ctx)

"""sort_particles! with cells from positions (grid_sorting.jl:58-113)."""
sort_particles!(grid::DeviceGrid1D, dp::DeviceParticles, species) =
    check(ccall((:mz_sort, libmz), Cint, (Ptr{Cvoid}, Int32, Ref{DeviceGrid1D}, Ptr{Int64}),
                dp.ptr, species - 1, grid, C_NULL), dp.ctx)

"""sort_particles! with cells stored by convection (grid_sorting.jl:128-182)."""
sort_particles!(dp::DeviceParticles, species) =
    check(ccall((:mz_sort, libmz), Cint, (Ptr{Cvoid}, Int32, Ptr{DeviceGrid1D}, Ptr{Int64}),
                dp.ptr, species - 1, C_NULL, C_NULL), dp.ctx)

"""squash_pia! (particles.jl:622-701)."""
squash_pia!(dp::DeviceParticles, species) =
    check(ccall((:mz_squash, libmz), Cint, (Ptr{Cvoid}, Int32), dp.ptr, species - 1), dp.ctx)

# ------------------------------------------------------------------ properties
compute_props!(dp::DeviceParticles, p::DeviceProps) =
    check(ccall((:mz_compute_props, libmz), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int32), dp.ptr, p.ptr, MZ_PROPS_ALL), dp.ctx)
compute_props_sorted!(dp::DeviceParticles, p::DeviceProps) =
    check(ccall((:mz_compute_props, libmz), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int32), dp.ptr, p.ptr, MZ_PROPS_SORTED),
          dp.ctx)
compute_props_with_total_moments!(dp::DeviceParticles, p::DeviceProps) =
    check(ccall((:mz_compute_props, libmz), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int32), dp.ptr, p.ptr, MZ_PROPS_MOMENTS),
          dp.ctx)
avg_props!(avg::DeviceProps, inst::DeviceProps, n_avg_timesteps) =
    check(ccall((:mz_avg_props, libmz), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Float64), avg.ptr, inst.ptr, n_avg_timesteps),
          avg.dp.ctx)
clear_props!(p::DeviceProps) = check(ccall((:mz_clear_props, libmz), Cint, (Ptr{Cvoid},), p.ptr), p.dp.ctx)

"""Copy device properties into a Merzbild `PhysProps` (same array layouts)."""
function fetch!(phys_props, p::DeviceProps)
    lpa = Vector{Float64}(undef, p.dp.n_species)
    mom = p.n_moments > 0 ? phys_props.moments : C_NULL
    check(ccall((:mz_props_download, libmz), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                p.ptr, lpa, phys_props.np, phys_props.n, phys_props.v, phys_props.T, mom), p.dp.ctx)
    phys_props.lpa .= lpa
    phys_props
end

"""
    snapshot!(p::DeviceProps, slot, dst::Vector{Float64})

Start copying np, n, v, T (back to back, 6 n_cells n_species values) into
`dst` without stopping the device (`mz_props_snapshot`); the copy overlaps the
steps enqueued after it.  `dst` must stay alive until `snapshot_wait(p, slot)`.
With a `pinned_vector` the call returns at once; with ordinary (pageable)
memory the CUDA runtime completes the copy before returning.
"""
snapshot!(p::DeviceProps, slot, dst::Vector{Float64}) =
    check(ccall((:mz_props_snapshot, libmz), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), p.ptr, slot, dst), p.dp.ctx)
snapshot_wait(p::DeviceProps, slot) =
    check(ccall((:mz_props_snapshot_wait, libmz), Cint, (Ptr{Cvoid}, Int32), p.ptr, slot), p.dp.ctx)

"""A page-locked `Vector{Float64}` of length n (`mz_host_alloc`); release it
with `free_pinned!`."""
function pinned_vector(ctx::DeviceContext, n::Integer)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:mz_host_alloc, libmz), Cint, (Ptr{Cvoid}, Csize_t, Ref{Ptr{Cvoid}}), ctx.ptr, n * 8, r), ctx)
    unsafe_wrap(Vector{Float64}, Ptr{Float64}(r[]), n; own=false)
end
free_pinned!(v::Vector{Float64}) = ccall((:mz_host_free, libmz), Cint, (Ptr{Cvoid},), pointer(v))

"""Copy a snapshot's values into a Merzbild `PhysProps` (np, n, v, T)."""
function unpack_snapshot!(phys_props, flat::Vector{Float64})
    m = length(phys_props.np)
    copyto!(phys_props.np, 1, flat, 1, m)
    copyto!(phys_props.n, 1, flat, m + 1, m)
    copyto!(phys_props.v, 1, flat, 2m + 1, 3m)
    copyto!(phys_props.T, 1, flat, 5m + 1, m)
    phys_props
end

# ------------------------------------------------------------------ merging and sampling
"""merge_octree_N2_based! (merging_octree_N2.jl:1060, :1088) for a cell or a
range of cells; `threshold` merges only cells with more particles."""
function merge_octree_N2_based!(rng::DeviceRNG, octree::DeviceOctree, dp::DeviceParticles, cell, species, target_np;
                                grid::Union{Nothing,DeviceGrid1D}=nothing, threshold=-1)
    cb, ce = cellrange(cell)
    n = Ref{Int64}(0)
    if grid === nothing
        check(ccall((:mz_merge_octree_n2, libmz), Cint,
                    (Ptr{Cvoid}, Int32, Int64, Int64, Int64, Int64, Ref{DeviceOctree}, Ptr{DeviceGrid1D}, UInt64,
                     Ref{Int64}), dp.ptr, species - 1, cb, ce, threshold, target_np, octree, C_NULL, rng.step, n),
              dp.ctx)
    else
        check(ccall((:mz_merge_octree_n2, libmz), Cint,
                    (Ptr{Cvoid}, Int32, Int64, Int64, Int64, Int64, Ref{DeviceOctree}, Ref{DeviceGrid1D}, UInt64,
                     Ref{Int64}), dp.ptr, species - 1, cb, ce, threshold, target_np, octree, grid, rng.step, n),
              dp.ctx)
    end
    n[]
end

"""sample_particles_equal_weight!(rng, grid, ..., ndens, T, Fnum; vx0, vy0, vz0) (grid_uniform1D.jl:198-219)."""
sample_particles_equal_weight!(rng::DeviceRNG, grid::DeviceGrid1D, dp::DeviceParticles, species, ndens, T, Fnum;
                               vx0=0.0, vy0=0.0, vz0=0.0) =
    check(ccall((:mz_sample_grid_ndens, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ref{DeviceGrid1D}, Float64, Float64, Float64, UInt64, Ptr{Float64}),
                dp.ptr, species - 1, grid, ndens, T, Fnum, rng.step, Float64[vx0, vy0, vz0]), dp.ctx)

"""sample_particles_equal_weight!(rng, particles, pia, cell, species, nparticles, m, T, Fnum, xlo, xhi, ylo,
yhi, zlo, zhi; distribution, vx0, vy0, vz0) (distributions_and_sampling.jl:477-509) for one cell."""
function sample_particles_equal_weight!(rng::DeviceRNG, dp::DeviceParticles, cell, species, nparticles, T, Fnum,
                                        xlo, xhi, ylo, yhi, zlo, zhi; distribution=:Maxwellian, vx0=0.0, vy0=0.0,
                                        vz0=0.0)
    counts = zeros(Int64, dp.n_cells)
    counts[cell] = nparticles
    Fn = fill(Float64(Fnum), dp.n_cells)
    box = zeros(6, dp.n_cells)
    box[:, cell] .= (xlo, xhi, ylo, yhi, zlo, zhi)
    check(ccall((:mz_sample_cells, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64, Ptr{Float64},
                 Int32, UInt64, Ptr{Float64}, Ptr{Float64}),
                dp.ptr, species - 1, counts, C_NULL, Float64[T, T, T], Fn, 0.0, box,
                distribution == :BKW ? 1 : 0, rng.step, C_NULL, Float64[vx0, vy0, vz0]), dp.ctx)
end

# ------------------------------------------------------------------ fused steps
"""
    step!(dp, n_steps; grid, walls, Δt, step0, inst, avg, avg_start, n_avg, dims,
          equal_weight, merge_threshold, merge_target, octree)

`n_steps` fused steps replayed from a CUDA graph: with `equal_weight=true`
ntc_equal_weight! -> convect -> sort -> props -> avg_props!, the loop body of
simulations/1D/couette_benchmarking.jl:58-85; with `equal_weight=false` ntc!
with splitting and the octree merge of cells above `merge_threshold`
particles down to `merge_target` before convection, the loop body of
simulations/1D/couette_varweight_octree.jl:85-135.  `dims=0` runs 0-D cells
(no convection).
"""
function step!(dp::DeviceParticles, n_steps; grid::DeviceGrid1D=DeviceGrid1D(1.0, dp.n_cells, 1.0, 1.0, 0.0, 1.0),
               walls::Union{Nothing,DeviceWalls1D}=nothing, Δt, step0=0,
               inst::Union{Nothing,DeviceProps}=nothing, avg::Union{Nothing,DeviceProps}=nothing,
               avg_start=0, n_avg=1, dims=1, equal_weight=true, merge_threshold=0, merge_target=0,
               octree::DeviceOctree=DeviceOctree(), dw_tol=1e-16)
    w = walls === nothing ? DeviceWalls1D((0.0, 0.0), ntuple(_ -> 0.0, 6), (0.0, 0.0),
                                          ntuple(_ -> 0.0, 2 * MZ_MAX_SPECIES)) : walls
    plan = MzStepPlan(dims, 1, equal_weight ? 1 : 0, 1, avg_start, n_avg, Δt, dw_tol, step0, 1, 0, grid, w, 0, 0,
                      merge_threshold, merge_target, octree, 0)
    check(ccall((:mz_step, libmz), Cint, (Ptr{Cvoid}, Ref{MzStepPlan}, Int64, Ptr{Cvoid}, Ptr{Cvoid}),
                dp.ptr, plan, n_steps, inst === nothing ? C_NULL : inst.ptr, avg === nothing ? C_NULL : avg.ptr),
          dp.ctx)
end

# ------------------------------------------------------------------ surface properties
mutable struct DeviceSurfProps
    dp::DeviceParticles
    ptr::Ptr{Cvoid}
end

"""
    DeviceSurfProps(dp)

Device counterpart of `SurfProps(pia, grid)` for a 1-D grid
(surface_props.jl:22-67): element 1 = left wall, element 2 = right wall.
"""
function DeviceSurfProps(dp::DeviceParticles)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:mz_surf_props_create, libmz), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}), dp.ptr, r), dp.ctx)
    sp = DeviceSurfProps(dp, r[])
    finalizer(q -> ccall((:mz_surf_props_destroy, libmz), Cint, (Ptr{Cvoid},), q.ptr), sp)
    sp
end

"""convect_particles! with surface sampling (convection_1D.jl:176-206)."""
convect_particles!(rng::DeviceRNG, grid::DeviceGrid1D, walls::DeviceWalls1D, dp::DeviceParticles, species,
                   surf::DeviceSurfProps, Δt) =
    check(ccall((:mz_convect_1d_surf, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ref{DeviceGrid1D}, Ref{DeviceWalls1D}, Float64, UInt64, Int32, Ptr{Cvoid}),
                dp.ptr, species - 1, grid, walls, Δt, rng.step, 0, surf.ptr), dp.ctx)
clear_props!(sp::DeviceSurfProps) =
    check(ccall((:mz_surf_props_clear, libmz), Cint, (Ptr{Cvoid},), sp.ptr), sp.dp.ctx)
avg_props!(avg::DeviceSurfProps, inst::DeviceSurfProps, n_avg_timesteps) =
    check(ccall((:mz_surf_avg_props, libmz), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Float64), avg.ptr, inst.ptr,
                n_avg_timesteps), avg.dp.ctx)

"""Copy device surface properties into a Merzbild `SurfProps` (same layouts)."""
function fetch!(surf_props, sp::DeviceSurfProps)
    check(ccall((:mz_surf_props_download, libmz), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                 Ptr{Float64}), sp.ptr, surf_props.np, surf_props.flux_incident, surf_props.flux_reflected,
                surf_props.force, surf_props.normal_pressure, surf_props.shear_pressure,
                surf_props.kinetic_energy_flux), sp.dp.ctx)
    surf_props
end

"""Sample the walls in every fused step (clear, sample, scale; `avg` averaged like avg_props!)."""
set_step_surface!(dp::DeviceParticles, inst::Union{Nothing,DeviceSurfProps},
                  avg::Union{Nothing,DeviceSurfProps}=nothing) =
    check(ccall((:mz_step_set_surface, libmz), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}), dp.ptr,
                inst === nothing ? C_NULL : inst.ptr, avg === nothing ? C_NULL : avg.ptr), dp.ctx)

# ------------------------------------------------------------------ netCDF output
struct MzNcAttribute
    name::Cstring
    type::Int32
    count::Int32
    values::Ptr{Cvoid}
end

mutable struct DeviceNCDataHolder
    ptr::Ptr{Cvoid}
    ctx::DeviceContext
end

function nc_check(rc, f::Ptr{Cvoid}, ctx)
    rc == 0 && return nothing
    if f != C_NULL
        buf = Vector{UInt8}(undef, 1024)
        ccall((:mz_nc_last_error, libmz), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), f, buf, length(buf))
        throw(ErrorException(unsafe_string(pointer(buf))))
    end
    check(rc, ctx)
end

# global attributes as text, Int32 or Float64 arrays (the values stay referenced in `keep`)
function nc_attributes(global_attributes, keep)
    atts = MzNcAttribute[]
    for (k, v) in global_attributes
        name = Base.cconvert(Cstring, string(k)); push!(keep, name)
        if v isa AbstractString
            data = Vector{UInt8}(codeunits(v)); t = Int32(0)
        elseif eltype(v) <: Integer
            data = Int32.(collect(v)); t = Int32(1)
        else
            data = Float64.(collect(v)); t = Int32(2)
        end
        push!(keep, data)
        push!(atts, MzNcAttribute(Base.unsafe_convert(Cstring, name), t, length(data), pointer(data)))
    end
    atts
end

"""
    DeviceNCDataHolder(nc_filename, names_skip_list, species_data, p::DeviceProps; global_attributes=Dict())

`NCDataHolder` (io.jl:143-224) whose records are written from device
properties; the layout is the reference's (netCDF classic container).
"""
function DeviceNCDataHolder(nc_filename, names_skip_list, species_data, p::DeviceProps;
                            global_attributes=Dict{Any,Any}())
    keep = Any[]
    atts = nc_attributes(global_attributes, keep)
    powers = Int32.(p.moment_powers)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep begin
        check(ccall((:mz_nc_props_create, libmz), Cint,
                    (Cstring, Ptr{Cstring}, Int32, Ptr{Cstring}, Int32, Int32, Int32, Int32, Ptr{Int32}, Int32,
                     Ptr{MzNcAttribute}, Int32, Ptr{Cvoid}, Ref{Ptr{Cvoid}}),
                    nc_filename, String.(names_skip_list), length(names_skip_list), [s.name for s in species_data],
                    length(species_data), p.dp.n_species, p.dp.n_cells, length(powers), powers,
                    p.ndens_not_Np ? 1 : 0, atts, length(atts), p.dp.ctx.ptr, r), p.dp.ctx)
    end
    ds = DeviceNCDataHolder(r[], p.dp.ctx)
    finalizer(close_netcdf, ds)
    ds
end
DeviceNCDataHolder(nc_filename, species_data, p::DeviceProps; global_attributes=Dict{Any,Any}()) =
    DeviceNCDataHolder(nc_filename, String[], species_data, p; global_attributes=global_attributes)

"""`NCDataHolderSurf` (io.jl:457-527) for device surface properties."""
function DeviceNCDataHolderSurf(nc_filename, names_skip_list, species_data, sp::DeviceSurfProps;
                                global_attributes=Dict{Any,Any}())
    keep = Any[]
    atts = nc_attributes(global_attributes, keep)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep begin
        check(ccall((:mz_nc_surf_create, libmz), Cint,
                    (Cstring, Ptr{Cstring}, Int32, Ptr{Cstring}, Int32, Int32, Int32, Ptr{MzNcAttribute}, Int32,
                     Ptr{Cvoid}, Ref{Ptr{Cvoid}}),
                    nc_filename, String.(names_skip_list), length(names_skip_list), [s.name for s in species_data],
                    length(species_data), sp.dp.n_species, 2, atts, length(atts), sp.dp.ctx.ptr, r), sp.dp.ctx)
    end
    ds = DeviceNCDataHolder(r[], sp.dp.ctx)
    finalizer(close_netcdf, ds)
    ds
end
DeviceNCDataHolderSurf(nc_filename, species_data, sp::DeviceSurfProps; global_attributes=Dict{Any,Any}()) =
    DeviceNCDataHolderSurf(nc_filename, String[], species_data, sp; global_attributes=global_attributes)

"""write_netcdf(ds, phys_props, timestep; sync_freq) (io.jl:274-317), enqueued
behind the device work; the library's writer thread writes the record."""
write_netcdf(ds::DeviceNCDataHolder, p::DeviceProps, timestep; sync_freq=0) =
    nc_check(ccall((:mz_nc_props_write, libmz), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Float64, Int32),
                   ds.ptr, p.ptr, timestep, sync_freq), ds.ptr, ds.ctx)

"""write_netcdf(ds, surf_props, timestep; sync_freq) (io.jl:566-603)."""
write_netcdf(ds::DeviceNCDataHolder, sp::DeviceSurfProps, timestep; sync_freq=0) =
    nc_check(ccall((:mz_nc_surf_write, libmz), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Float64, Int32),
                   ds.ptr, sp.ptr, timestep, sync_freq), ds.ptr, ds.ctx)

"""close_netcdf(ds) (io.jl:251-253): writes what is enqueued, then closes."""
function close_netcdf(ds::DeviceNCDataHolder)
    ds.ptr == C_NULL && return nothing
    p, ds.ptr = ds.ptr, C_NULL
    rc = ccall((:mz_nc_close, libmz), Cint, (Ptr{Cvoid},), p)
    rc == 0 || throw(ErrorException("netCDF file could not be completed"))
    nothing
end

function counters(dp::DeviceParticles; reset=false)
    c = Ref{MzCounters}()
    check(ccall((:mz_get_counters, libmz), Cint, (Ptr{Cvoid}, Ref{MzCounters}, Int32), dp.ptr, c, reset), dp.ctx)
    c[]
end

# ------------------------------------------------------------------ serving
# Continuous batching of independent 0-D relaxation requests (mz_server_*);
# no reference counterpart: each request is the README's 0-D loop.
struct MzRequest
    count::NTuple{MZ_MAX_SPECIES,Int64}
    T::NTuple{MZ_MAX_SPECIES,Float64}
    Fnum::Float64
    V::Float64
    n_steps::Int64
    seed::UInt64
end

struct MzRequestResult
    id::Int64
    state::Int32
    reserved::Int32
    steps_done::Int64
    np::NTuple{MZ_MAX_SPECIES,Int64}
    n::NTuple{MZ_MAX_SPECIES,Float64}
    v::NTuple{3 * MZ_MAX_SPECIES,Float64}  # species-major: v[3(s-1) + k]
    T::NTuple{MZ_MAX_SPECIES,Float64}
end

mutable struct DeviceServer
    ctx::DeviceContext
    ptr::Ptr{Cvoid}
    n_species::Int
end

"""
    DeviceServer(ctx, species_data, interactions, Δt, max_requests, capacity)

A server for up to `max_requests` concurrent requests with `capacity`
particles of each species in device memory.
"""
function DeviceServer(ctx::DeviceContext, species_data, interactions, Δt, max_requests, capacity)
    ns = length(species_data)
    tab = [MzInteraction(interactions[s1, s2].m_r, interactions[s1, s2].μ1, interactions[s1, s2].μ2,
                         interactions[s1, s2].vhs_d, interactions[s1, s2].vhs_o, interactions[s1, s2].vhs_Tref,
                         interactions[s1, s2].vhs_muref, interactions[s1, s2].vhs_factor) for s1 in 1:ns, s2 in 1:ns]
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:mz_server_create, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{MzInteraction}, Float64, Int64, Ptr{Int64}, Ref{Ptr{Cvoid}}),
                ctx.ptr, ns, [s.mass for s in species_data], tab, Δt, max_requests, fill(Int64(capacity), ns), r),
          ctx)
    srv = DeviceServer(ctx, r[], ns)
    finalizer(v -> ccall((:mz_server_destroy, libmz), Cint, (Ptr{Cvoid},), v.ptr), srv)
    srv
end

"""Queue a request (particles and temperature per species); returns its id."""
function submit!(srv::DeviceServer, counts, T, Fnum, n_steps, seed; V=1.0)
    pad(a, z) = ntuple(i -> i <= length(a) ? a[i] : z, MZ_MAX_SPECIES)
    req = MzRequest(pad(Int64.(counts), Int64(0)), pad(Float64.(T), 0.0), Fnum, V, n_steps, UInt64(seed))
    id = Ref{Int64}(0)
    check(ccall((:mz_server_submit, libmz), Cint, (Ptr{Cvoid}, Ref{MzRequest}, Ref{Int64}), srv.ptr, req, id),
          srv.ctx)
    id[]
end

"""Admit, run up to `max_steps` steps, retire; returns (running, queued, retired)."""
function server_step!(srv::DeviceServer; max_steps=16)
    k, run, que, ret = Ref{Int64}(0), Ref{Int64}(0), Ref{Int64}(0), Ref{Int64}(0)
    check(ccall((:mz_server_step_many, libmz), Cint,
                (Ptr{Cvoid}, Int64, Ref{Int64}, Ref{Int64}, Ref{Int64}, Ref{Int64}), srv.ptr, max_steps, k, run, que,
                ret), srv.ctx)
    (run[], que[], ret[])
end

"""State of request `id` and, once done, compute_props! of its last step."""
function request_result(srv::DeviceServer, id)
    r = Ref{MzRequestResult}()
    check(ccall((:mz_server_result, libmz), Cint, (Ptr{Cvoid}, Int64, Ref{MzRequestResult}), srv.ptr, id, r),
          srv.ctx)
    x, ns = r[], srv.n_species
    (state=x.state, steps_done=x.steps_done, np=collect(x.np[1:ns]), n=collect(x.n[1:ns]),
     v=[x.v[3 * (s - 1) + k] for k in 1:3, s in 1:ns], T=collect(x.T[1:ns]))
end

"""Ids of the requests the last server_step! retired."""
function retired_requests(srv::DeviceServer)
    n = Ref{Int64}(0)
    check(ccall((:mz_server_retired, libmz), Cint, (Ptr{Cvoid}, Int64, Ptr{Int64}, Ref{Int64}), srv.ptr, 0,
                C_NULL, n), srv.ctx)
    ids = zeros(Int64, n[])
    check(ccall((:mz_server_retired, libmz), Cint, (Ptr{Cvoid}, Int64, Ptr{Int64}, Ref{Int64}), srv.ptr, n[],
                ids, n), srv.ctx)
    ids
end

# ------------------------------------------------------------------ the reference's signatures
# Stand-ins for the reference's containers.  A time loop written against
# Merzbild (simulations/**, test/**) keeps its calls and their positional
# arguments; only the set-up builds device containers:
#
#     dp = DeviceParticles(ctx, grid, species_data, interaction_data, capacity)
#     particles = device_particles(dp); pia = DevicePIA(dp)
#     collision_factors = create_collision_factors_array(pia, interaction_data, species_data, T, Fnum)
#     gridsorter = DeviceGridSort(dp); rng = DeviceRNG(seed)
#     ... then the reference's loop body, e.g. couette_benchmarking.jl:58-85:
#     ntc_equal_weight!(rng, collision_factors[1, 1, cell], collision_data, interaction_data,
#                       particles[1], pia, cell, 1, Δt, grid.cells[cell].V)
#
# Arguments the device keeps for itself (collision_data scratch, the
# interaction, which the domain was created with) are accepted and unused.

"""
    DevicePIA(dp)

`ParticleIndexerArray` (particles.jl:110-141) of a `DeviceParticles`: the
indexers live on the device.
"""
struct DevicePIA
    dp::DeviceParticles
end

"""
    DeviceParticleVector(dp, species)

`ParticleVector` (particles.jl:194-212) of one species of a `DeviceParticles`.
"""
struct DeviceParticleVector
    dp::DeviceParticles
    species::Int
end

"""`particles[s]` for every species, as the reference's drivers index them."""
device_particles(dp::DeviceParticles) = [DeviceParticleVector(dp, s) for s in 1:dp.n_species]

"""
    DeviceCollisionFactors(dp)

The array of `CollisionFactors` (create_collision_factors_array,
collision_ntc.jl:46-155) of a `DeviceParticles`; `cf[s1, s2, cell]` is the
handle the reference's `ntc!` takes, the factors stay on the device.
"""
struct DeviceCollisionFactors
    dp::DeviceParticles
end
struct DeviceCollisionFactorsCell
    dp::DeviceParticles
    species1::Int
    species2::Int
    cell::Int
end
Base.getindex(cf::DeviceCollisionFactors, s1::Integer, s2::Integer, cell::Integer) =
    DeviceCollisionFactorsCell(cf.dp, s1, s2, cell)
Base.size(cf::DeviceCollisionFactors) = (cf.dp.n_species, cf.dp.n_species, cf.dp.n_cells)

"""`GridSortInPlace` (grid_sorting.jl:10-27): the device sort keeps its buffers on the device."""
struct DeviceGridSort
    dp::DeviceParticles
end

"""
    DeviceParticles(ctx, grid, species_data, interactions, capacity; seed=1234)

A `DeviceParticles` on the cells of a 1-D grid, with the grid's cell volumes.
"""
function DeviceParticles(ctx::DeviceContext, grid::Merzbild.Grid1DUniform, species_data, interactions, capacity;
                         seed=1234)
    dp = DeviceParticles(ctx, grid.n_cells, species_data, interactions, capacity; seed=seed)
    set_cell_volumes!(dp, [c.V for c in grid.cells])
    dp
end

function same_domain(dp::DeviceParticles, others...)
    for o in others
        o.dp === dp || throw(ErrorException("device containers of different DeviceParticles"))
    end
    dp
end

function check_volume(dp::DeviceParticles, cell, V)
    dp.V[cell] == V || throw(ErrorException("cell $cell: volume $V differs from the device's $(dp.V[cell]); " *
                                            "set the volumes with set_cell_volumes! or DeviceParticles(ctx, grid, ...)"))
end

device_grid(grid::DeviceGrid1D) = grid
device_grid(grid::Merzbild.Grid1DUniform) = DeviceGrid1D(grid)
device_walls(walls::DeviceWalls1D) = walls
device_walls(walls::Merzbild.MaxwellWalls1D) = DeviceWalls1D(walls)

function ntc_call(rng::DeviceRNG, kind::Symbol, cf::DeviceCollisionFactorsCell, pia::DevicePIA, cell, s1, s2, Δt, V,
                  flags, dw_tol)
    dp = same_domain(pia.dp, cf)
    (cf.species1 == s1 && cf.species2 == s2 && cf.cell == cell) ||
        throw(ErrorException("collision factors of species ($(cf.species1), $(cf.species2)), cell $(cf.cell) " *
                             "passed for species ($s1, $s2), cell $cell"))
    check_volume(dp, cell, V)
    step = drop_in_step!(rng, kind, s1, s2, cell)
    check(ccall((:mz_ntc, libmz), Cint, (Ptr{Cvoid}, Int32, Int32, Float64, Int64, Int64, UInt64, Int32, Float64),
                dp.ptr, s1 - 1, s2 - 1, Δt, cell - 1, cell, step, flags, dw_tol), dp.ctx)
end

"""ntc! of one species (collision_ntc.jl:338)."""
Merzbild.ntc!(rng::DeviceRNG, collision_factors::DeviceCollisionFactorsCell, collision_data, interaction,
              particles::DeviceParticleVector, pia::DevicePIA, cell, species, Δt, V; dw_tol=1e-16) =
    ntc_call(rng, :ntc, collision_factors, same_pv(pia, particles), cell, species, species, Δt, V, 0, dw_tol)

"""ntc! of two species (collision_ntc.jl:412)."""
Merzbild.ntc!(rng::DeviceRNG, collision_factors::DeviceCollisionFactorsCell, collision_data, interaction,
              particles_1::DeviceParticleVector, particles_2::DeviceParticleVector, pia::DevicePIA,
              cell, species1, species2, Δt, V; dw_tol=1e-16) =
    ntc_call(rng, :ntc, collision_factors, same_pv(pia, particles_1, particles_2), cell, species1, species2, Δt, V,
             0, dw_tol)

"""ntc_equal_weight! of one species (collision_ntc.jl:479)."""
Merzbild.ntc_equal_weight!(rng::DeviceRNG, collision_factors::DeviceCollisionFactorsCell, collision_data,
                           interaction, particles::DeviceParticleVector, pia::DevicePIA, cell, species, Δt, V) =
    ntc_call(rng, :ntc, collision_factors, same_pv(pia, particles), cell, species, species, Δt, V,
             MZ_NTC_EQUAL_WEIGHT, 1e-16)

"""ntc_equal_weight! of two species (collision_ntc.jl:554)."""
Merzbild.ntc_equal_weight!(rng::DeviceRNG, collision_factors::DeviceCollisionFactorsCell, collision_data,
                           interaction, particles_1::DeviceParticleVector, particles_2::DeviceParticleVector,
                           pia::DevicePIA, cell, species1, species2, Δt, V) =
    ntc_call(rng, :ntc, collision_factors, same_pv(pia, particles_1, particles_2), cell, species1, species2, Δt,
             V, MZ_NTC_EQUAL_WEIGHT, 1e-16)

function same_pv(pia::DevicePIA, pvs::DeviceParticleVector...)
    same_domain(pia.dp, pvs...)
    pia
end

"""create_collision_factors_array(pia) (collision_ntc.jl:93): the device's
collision factors of every pair and cell, (σ g w)_max as last set."""
Merzbild.create_collision_factors_array(pia::DevicePIA) = DeviceCollisionFactors(pia.dp)

"""create_collision_factors_array(pia, interactions, species_data, T_list, Fnum; mult_factor)
(collision_ntc.jl:120): (σ g w)_max of every pair in every cell, estimated as
the reference does (estimate_sigma_g_w_max!, collision_utils.jl:464-478)."""
function Merzbild.create_collision_factors_array(pia::DevicePIA, interactions, species_data, T_list, Fnum::Real;
                                                 mult_factor=1.0)
    dp = pia.dp
    for (k, species2) in enumerate(species_data), (i, species1) in enumerate(species_data)
        v = Merzbild.estimate_sigma_g_w_max(interactions[i, k], species1, species2, T_list[i], T_list[k], Fnum;
                                            mult_factor=mult_factor)
        set_sigma_g_w_max!(dp, i, k, fill(v, dp.n_cells))
    end
    DeviceCollisionFactors(dp)
end
Merzbild.create_collision_factors_array(pia::DevicePIA, interactions, species_data, T::Real, Fnum::Real;
                                        mult_factor=1.0) =
    Merzbild.create_collision_factors_array(pia, interactions, species_data, fill(T, length(species_data)), Fnum;
                                            mult_factor=mult_factor)

"""compute_props! (physical_props.jl:104)."""
Merzbild.compute_props!(particles::AbstractVector{DeviceParticleVector}, pia::DevicePIA, species_data,
                        phys_props::DeviceProps) = compute_props!(same_pv(pia, particles...).dp, phys_props)

"""compute_props_with_total_moments! (physical_props.jl:168)."""
Merzbild.compute_props_with_total_moments!(particles::AbstractVector{DeviceParticleVector}, pia::DevicePIA,
                                           species_data, phys_props::DeviceProps) =
    compute_props_with_total_moments!(same_pv(pia, particles...).dp, phys_props)

"""compute_props_sorted! (physical_props.jl:370; every cell) and its grid
forms (:393, :452), number densities when `phys_props` computes them.  The
forms with a `cell_chunk` (:317, :393; the reference's threads each take a
chunk) compute every cell at once on the device: the chunk's cells get the
values the reference computes, the other cells are recomputed from the same
state."""
Merzbild.compute_props_sorted!(particles::AbstractVector{DeviceParticleVector}, pia::DevicePIA, species_data,
                               phys_props::DeviceProps) = compute_props_sorted!(same_pv(pia, particles...).dp, phys_props)
Merzbild.compute_props_sorted!(particles::AbstractVector{DeviceParticleVector}, pia::DevicePIA, species_data,
                               phys_props::DeviceProps, cell_chunk) =
    compute_props_sorted!(same_pv(pia, particles...).dp, phys_props)
Merzbild.compute_props_sorted!(particles::AbstractVector{DeviceParticleVector}, pia::DevicePIA, species_data,
                               phys_props::DeviceProps, grid::Merzbild.Grid1DUniform) =
    compute_props_sorted!(same_pv(pia, particles...).dp, phys_props)
Merzbild.compute_props_sorted!(particles::AbstractVector{DeviceParticleVector}, pia::DevicePIA, species_data,
                               phys_props::DeviceProps, grid::Merzbild.Grid1DUniform, cell_chunk) =
    compute_props_sorted!(same_pv(pia, particles...).dp, phys_props)

"""convect_particles! (convection_1D.jl:130) and with surface sampling (:176)."""
function Merzbild.convect_particles!(rng::DeviceRNG, grid, boundaries, particles::DeviceParticleVector,
                                     pia::DevicePIA, species, species_data, Δt)
    dp = same_pv(pia, particles).dp
    step = drop_in_step!(rng, :convect, species, species, 1)
    check(ccall((:mz_convect_1d, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ref{DeviceGrid1D}, Ref{DeviceWalls1D}, Float64, UInt64, Int32),
                dp.ptr, species - 1, device_grid(grid), device_walls(boundaries), Δt, step, 0), dp.ctx)
end
function Merzbild.convect_particles!(rng::DeviceRNG, grid, boundaries, particles::DeviceParticleVector,
                                     pia::DevicePIA, species, species_data, surf_props::DeviceSurfProps, Δt)
    dp = same_pv(pia, particles).dp
    step = drop_in_step!(rng, :convect, species, species, 1)
    check(ccall((:mz_convect_1d_surf, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ref{DeviceGrid1D}, Ref{DeviceWalls1D}, Float64, UInt64, Int32, Ptr{Cvoid}),
                dp.ptr, species - 1, device_grid(grid), device_walls(boundaries), Δt, step, 0, surf_props.ptr), dp.ctx)
end

"""sort_particles!(gridsort, grid, particles, pia, species) (grid_sorting.jl:58)
and without the grid, from the cells stored in the particles (:128)."""
Merzbild.sort_particles!(gridsort::DeviceGridSort, grid, particles::DeviceParticleVector, pia::DevicePIA, species) =
    sort_particles!(device_grid(grid), same_pv(pia, particles).dp, species)
Merzbild.sort_particles!(gridsort::DeviceGridSort, particles::DeviceParticleVector, pia::DevicePIA, species) =
    sort_particles!(same_pv(pia, particles).dp, species)

"""merge_octree_N2_based!(rng, octree, particles, pia, cell, species, target_np[, grid])
(merging_octree_N2.jl:1060, :1088)."""
function Merzbild.merge_octree_N2_based!(rng::DeviceRNG, octree::DeviceOctree, particles::DeviceParticleVector,
                                         pia::DevicePIA, cell, species, target_np)
    step = drop_in_step!(rng, :merge, species, species, cell)
    merge_octree_N2_based!(DeviceRNG(rng.seed, step), octree, same_pv(pia, particles).dp, cell, species, target_np)
end
function Merzbild.merge_octree_N2_based!(rng::DeviceRNG, octree::DeviceOctree, particles::DeviceParticleVector,
                                         pia::DevicePIA, cell, species, target_np, grid::Merzbild.Grid1DUniform)
    step = drop_in_step!(rng, :merge, species, species, cell)
    merge_octree_N2_based!(DeviceRNG(rng.seed, step), octree, same_pv(pia, particles).dp, cell, species, target_np;
                           grid=device_grid(grid))
end

"""squash_pia!(pv, pia, species) (particles.jl:622) and of every species (:695)."""
Merzbild.squash_pia!(pv::DeviceParticleVector, pia::DevicePIA, species) = squash_pia!(same_pv(pia, pv).dp, species)
function Merzbild.squash_pia!(particles::AbstractVector{DeviceParticleVector}, pia::DevicePIA)
    dp = same_pv(pia, particles...).dp
    for s in 1:dp.n_species
        squash_pia!(dp, s)
    end
end

"""The reference's indexing checks (particles.jl:805-1025) on the device
layout: the same return values."""
function check_indexing(dp::DeviceParticles, species, mode)
    ok = Ref{Int32}(0)
    detail = Ref{Int64}(0)
    check(ccall((:mz_check_indexing, libmz), Cint, (Ptr{Cvoid}, Int32, Int32, Ref{Int32}, Ref{Int64}),
                dp.ptr, species - 1, mode, ok, detail), dp.ctx)
    ok[] != 0, detail[]
end
Merzbild.check_pia_is_correct(pia::DevicePIA, species) = check_indexing(pia.dp, species, 0)
Merzbild.check_unique_index(pv::DeviceParticleVector, pia::DevicePIA, species) =
    check_indexing(same_pv(pia, pv).dp, species, 1)
Merzbild.check_unique_buffer(pv::DeviceParticleVector) = check_indexing(pv.dp, pv.species, 2)
Merzbild.count_disordered_particles(pv::DeviceParticleVector, pia::DevicePIA, species; use_offset=true) =
    check_indexing(same_pv(pia, pv).dp, species, use_offset ? 3 : 4)[2]

"""Write a species' indexer rows as given (mz_set_indexer): 1-based
`ParticleIndexer`-like rows (n_local, start1, end1, n_group1, start2, end2,
n_group2), one per cell."""
function set_indexer!(dp::DeviceParticles, species, rows::AbstractMatrix{<:Integer}, n_total)
    tab = [MzParticleIndexer(rows[c, 1], rows[c, 4] > 0 ? rows[c, 2] - 1 : 0, rows[c, 4] > 0 ? rows[c, 3] - 1 : -1,
                             rows[c, 4], rows[c, 7] > 0 ? rows[c, 5] - 1 : 0, rows[c, 7] > 0 ? rows[c, 6] - 1 : -1,
                             rows[c, 7]) for c in 1:dp.n_cells]
    check(ccall((:mz_set_indexer, libmz), Cint, (Ptr{Cvoid}, Int32, Ptr{MzParticleIndexer}, Int64),
                dp.ptr, species - 1, tab, n_total), dp.ctx)
end

"""Requests of at least `particles` particles run in the lane of large requests (0: one lane)."""
set_lane_split!(srv::DeviceServer, particles) =
    check(ccall((:mz_server_set_lane_split, libmz), Cint, (Ptr{Cvoid}, Int64), srv.ptr, particles), srv.ctx)

"""Device memory that admission by free memory (a server created with capacity 0) leaves free."""
set_hbm_headroom!(srv::DeviceServer, bytes::Integer) =
    check(ccall((:mz_server_set_hbm_headroom, libmz), Cint, (Ptr{Cvoid}, Int64), srv.ptr, bytes), srv.ctx)

end # module
