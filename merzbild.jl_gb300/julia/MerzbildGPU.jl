"""
    MerzbildGPU

Julia binding of libmerzgpu.so (include/merzgpu.h): the per-step DSMC path of
Merzbild.jl (NTC collisions, 1-D convection, grid sorting, cell properties,
octree merging, sampling) on a GB300 GPU.

The module adds methods to Merzbild's own functions for a device-resident
particle type, so a time loop written against Merzbild keeps its calls and
swaps its particle containers:

    ctx = DeviceContext(0)
    dp  = DeviceParticles(ctx, n_cells, species_data, interactions, capacity)
    for t in 1:n_timesteps
        rng.step = t
        ntc_equal_weight!(rng, dp, (1, n_cells), 1, Δt)
        convect_particles!(rng, grid, walls, dp, 1, Δt)
        sort_particles!(grid, dp, 1)
        compute_props_sorted!(dp, props)
    end

Conventions at the boundary: the C ABI is 0-based (cells, slots); this
module takes and returns Merzbild's 1-based cells.  Random numbers come from
counter-based streams keyed on (seed, step, cell, particle), so `DeviceRNG`
carries a seed and the time-step index instead of a generator state.
"""
module MerzbildGPU

import Merzbild  # setup estimates (estimate_sigma_g_w_max) stay the reference's own

export DeviceContext, DeviceParticles, DeviceProps, DeviceRNG, DeviceGrid1D, DeviceWalls1D, DeviceOctree,
       upload!, download, ntc!, ntc_equal_weight!, convect_particles!, convect_particles_and_compute_cell!,
       sort_particles!, squash_pia!, compute_props!, compute_props_sorted!, compute_props_with_total_moments!,
       avg_props!, clear_props!, merge_octree_N2_based!, sample_particles_equal_weight!, step!, counters,
       DeviceSurfProps, set_step_surface!, DeviceNCDataHolder, DeviceNCDataHolderSurf, write_netcdf, close_netcdf,
       swpm!, create_collision_factors_swpm_array!, snapshot!, snapshot_wait, unpack_snapshot!, pinned_vector,
       free_pinned!, DeviceServer, submit!, server_step!, request_result, retired_requests, set_lane_split!

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
    dp = DeviceParticles(ctx, r[], n_cells, ns)
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

"""Seed and time-step index of the counter-based streams (replaces `rng`)."""
mutable struct DeviceRNG
    seed::UInt64
    step::UInt64
end
DeviceRNG(seed::Integer) = DeviceRNG(UInt64(seed), UInt64(0))

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

set_cell_volumes!(dp::DeviceParticles, V::Vector{Float64}) =
    check(ccall((:mz_set_cell_volumes, libmz), Cint, (Ptr{Cvoid}, Ptr{Float64}), dp.ptr, V), dp.ctx)

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

"""sample_particles_equal_weight!(rng, grid, ..., ndens, T, Fnum) (grid_uniform1D.jl:198-219)."""
sample_particles_equal_weight!(rng::DeviceRNG, grid::DeviceGrid1D, dp::DeviceParticles, species, ndens, T, Fnum) =
    check(ccall((:mz_sample_grid_ndens, libmz), Cint,
                (Ptr{Cvoid}, Int32, Ref{DeviceGrid1D}, Float64, Float64, Float64, UInt64),
                dp.ptr, species - 1, grid, ndens, T, Fnum, rng.step), dp.ctx)

# ------------------------------------------------------------------ fused steps
"""
    step!(dp, n_steps; grid, walls, Δt, step0, inst, avg, avg_start, n_avg)

`n_steps` fused steps (ntc_equal_weight! -> convect -> sort -> props ->
avg_props!), replayed from a CUDA graph: the loop body of
simulations/1D/couette_benchmarking.jl:58-85 in one call.
"""
function step!(dp::DeviceParticles, n_steps; grid::DeviceGrid1D, walls::DeviceWalls1D, Δt, step0=0,
               inst::Union{Nothing,DeviceProps}=nothing, avg::Union{Nothing,DeviceProps}=nothing,
               avg_start=0, n_avg=1, dims=1)
    plan = MzStepPlan(dims, 1, 1, 1, avg_start, n_avg, Δt, 1e-16, step0, 1, 0, grid, walls, 0)
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

"""Requests of at least `particles` particles run in the lane of large requests (0: one lane)."""
set_lane_split!(srv::DeviceServer, particles) =
    check(ccall((:mz_server_set_lane_split, libmz), Cint, (Ptr{Cvoid}, Int64), srv.ptr, particles), srv.ctx)

end # module
