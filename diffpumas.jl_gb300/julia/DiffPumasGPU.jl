# DiffPumasGPU.jl -- the ccall layer a DiffPumas.jl host adds to route the hot
# path (run_backward_mc, compute_flux, compute_flux_differentiable, the MIXED
# kernels, the batched and directional MC, the voxel tomography forward model
# and J^T r, the water-fraction CSDA operator and the device inversion loops)
# to libdpgpu.so through its C ABI (include/dpgpu.h).
#
# Every struct passed by reference mirrors the C struct of the same name
# (DpFoo <-> dp_foo): field names, order and C types.  tests/test_julia_layout.py
# checks that on the CPU, and that every ccall names a symbol the header
# declares.  Handles (contexts, tables, mixtures, paths) own their device
# memory and free it from finalizers.
module DiffPumasGPU

using DiffPumas, ChainRulesCore, SparseArrays

const lib = joinpath(@__DIR__, "..", "_build", "libdpgpu.so")

# ---------------------------------------------------------------- structs
struct DpSettings
    mass::Cdouble; ctau::Cdouble; cutoff::Cdouble; elastic_ratio::Cdouble
end
struct DpElement
    Z::Cdouble; A::Cdouble; I::Cdouble; fraction::Cdouble
end
struct DpMaterial
    name::Cstring; density::Cdouble; I::Cdouble; ZoA::Cdouble
    n_elements::Cint; elements::Ptr{DpElement}
end
struct DpMcParams
    rock_thickness::Cdouble; rock_density::Cdouble; elevation::Cdouble
    energy_min::Cdouble; energy_max::Cdouble; n_samples::Clong; seed::UInt64
    straggling::Cint; scattering::Cint; compute_gradient::Cint
    energy_threshold_low::Cdouble; source_energy_max::Cdouble; primary_altitude::Cdouble
    rock_material::Cint; air_material::Cint
    precision::Cint            # 0: the reference's FP64 operations; 1: mixed precision
    porous_material::Cint      # shallow porous layer (0-based; -1: none)
    porous_density::Cdouble; porous_thickness::Cdouble
end
struct DpMcResult
    flux::Cdouble; sigma::Cdouble; gradient::Cdouble; gradient_flux::Cdouble
    source_energy_max::Cdouble; n_samples::Clong; n_status_nonzero::Clong
end
struct DpMcConfig
    straggling::Cint; scattering::Cint; energy_threshold_low::Cdouble
    source_energy_max::Cdouble; seed::UInt64; precision::Cint
end
struct DpLos
    thickness::Cdouble; thickness_max::Cdouble; density::Cdouble; density_max::Cdouble
    elevation::Cdouble; elevation_max::Cdouble; primary_altitude::Cdouble
    air_height::Cdouble; energy_min::Cdouble; energy_max::Cdouble; n_samples::Clong
    porous_thickness::Cdouble; porous_density::Cdouble
end
struct DpLosResult
    flux::Cdouble; sigma::Cdouble; gradient::Cdouble; gradient_flux::Cdouble
    n_samples::Clong; n_status_nonzero::Clong
end
struct DpDirBatch
    n_dirs::Clong; cos_theta::Ptr{Cdouble}; remaining_rock::Ptr{Cdouble}
    air_distance::Ptr{Cdouble}; valid::Ptr{Int32}; seg_ptr::Ptr{Int64}; seg_medium::Ptr{Int32}
    seg_density::Ptr{Cdouble}; seg_length::Ptr{Cdouble}; sample_ptr::Ptr{Int64}
    energy::Ptr{Cdouble}; charge::Ptr{Cdouble}; weight::Ptr{Cdouble}
    energy_min::Cdouble; energy_max::Cdouble; rock_medium::Cint; air_medium::Cint
    rock_density::Cdouble; detector_elevation::Cdouble
end
struct DpVoxelVolume
    nx::Cint; ny::Cint; nz::Cint
    x_edges::Ptr{Cdouble}; y_edges::Ptr{Cdouble}; z_edges::Ptr{Cdouble}
end
struct DpElevationMap
    nx::Cint; ny::Cint; x0::Cdouble; y0::Cdouble; dx::Cdouble; dy::Cdouble
    z::Ptr{Cdouble}            # z[iy*nx + ix]
end
struct DpTerrain
    map::DpElevationMap; xy_scale::Cdouble; detector_elevation::Cdouble
    step::Cdouble; max_distance::Cdouble
end
struct DpTetraMesh
    n_points::Clong; points::Ptr{Cdouble}; n_tets::Clong; tets::Ptr{Int32}
end
struct DpCsdaConfig
    rock_material::Cint; water_material::Cint; air_material::Cint; porous_material::Cint
    rock_density::Cdouble; water_density::Cdouble; porous_density::Cdouble
    porous_top_thickness::Cdouble; detector_elevation::Cdouble; primary_altitude::Cdouble
    correction::Cint; kappa_strag::Cdouble; kappa_hard::Cdouble
    resid_a::Cdouble; resid_b::Cdouble; resid_c::Cdouble; resid_d::Cdouble
    material_correction::Cint; material_linear::Cdouble; material_quadratic::Cdouble
end
struct DpCsdaBatch
    n_bins::Clong; cos_theta::Ptr{Cdouble}; remaining_rock::Ptr{Cdouble}
    surface_exit_z::Ptr{Cdouble}; valid::Ptr{Int32}; seg_ptr::Ptr{Int64}
    seg_cell::Ptr{Int32}; seg_length::Ptr{Cdouble}; n_energy::Cint
    energy::Ptr{Cdouble}; charge::Ptr{Cdouble}; weight::Ptr{Cdouble}
end
struct DpGrid
    nx::Cint; ny::Cint; nz::Cint; x0::Cdouble; y0::Cdouble; z0::Cdouble
    dx::Cdouble; dy::Cdouble; dz::Cdouble
end
struct DpRay
    ox::Cdouble; oy::Cdouble; oz::Cdouble; ux::Cdouble; uy::Cdouble; uz::Cdouble
    cos_theta::Cdouble
end
struct DpTomoParams
    rock_material::Cint; air_material::Cint; side_cell::Cint; side_density::Cdouble
    primary_altitude::Cdouble; n_nodes::Cint
    node_energy::Ptr{Cdouble}; node_charge::Ptr{Cdouble}; node_weight::Ptr{Cdouble}
    precision::Cint            # 0: FP64 parity, 1: mixed precision
end
struct DpSolveParams
    method::Cint; n_iter::Cint; cg_iter::Cint; precision::Cint
    relaxation::Cdouble; lm_damping::Cdouble; box_lo::Cdouble; box_hi::Cdouble
    prior_weight::Cdouble; smooth_strength::Cdouble; no_speculation::Cint
    optimizer::Cint; fixed_linearization::Cint; lr::Cdouble
end
struct DpMcShape
    threads::Cint; staging::Cint
    order::Cint                # 0: longest first, 1: index order
    sync::Cint                 # bit k: phase k steps in CTA lockstep
end

# ---------------------------------------------------------------- errors, context
last_error(ctx::Ptr{Cvoid}) = unsafe_string(ccall((:dp_last_error, lib), Cstring, (Ptr{Cvoid},), ctx))
# DP_ERR_ARG (-1) is an ArgumentError, DP_ERR_DOMAIN a DomainError carrying the
# reference's message; the rest are errors with the library's message
function check(rc::Integer, ctx::Ptr{Cvoid})
    rc == 0 && return nothing
    rc == -1 && throw(ArgumentError(last_error(ctx)))
    rc == -3 && throw(DomainError(nothing, last_error(ctx)))
    error(last_error(ctx))
end

mutable struct Context; h::Ptr{Cvoid}; end
function Context(device::Integer = 0)
    r = Ref{Ptr{Cvoid}}()
    ccall((:dp_init, lib), Cint, (Cint, Ref{Ptr{Cvoid}}), device, r) == 0 || error("dp_init failed")
    c = Context(r[])
    finalizer(c -> ccall((:dp_destroy, lib), Cint, (Ptr{Cvoid},), c.h), c)
end
# launch on a CUDA.jl stream: set_stream!(ctx, CUDA.stream().handle)
set_stream!(ctx::Context, stream::Ptr{Cvoid}) =
    check(ccall((:dp_set_stream, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), ctx.h, stream), ctx.h)

# ---------------------------------------------------------------- physics tables
# the tables built by DiffPumas.create_physics, handed to the device (the CPU
# tables stay the source of truth)
const COLS = (:energies, :log_energies, :csda_stopping_power, :csda_range, :csda_proper_time,
              :mixed_stopping_power, :mixed_range, :straggling, :ionization, :bremsstrahlung,
              :pair_production, :photonuclear, :cross_section, :transport_path, :elastic_path,
              :elastic_cutoff, :magnetic_rotation, :screening_parameter, :spin_factor)
mutable struct GPUPhysics; h::Ptr{Cvoid}; ctx::Context; end
function GPUPhysics(ctx::Context, h::Ptr{Cvoid})
    g = GPUPhysics(h, ctx)
    finalizer(g -> ccall((:dp_physics_free, lib), Cint, (Ptr{Cvoid},), g.h), g)
end
function upload(ctx::Context, p::DiffPumas.PhysicsTables)
    n = length(p.tables[1].energies)
    cols = Float64[]                                   # n_mat x 19 x n, row-major
    for t in p.tables, c in COLS
        append!(cols, getfield(t, c))
    end
    st = DpSettings(p.mass, p.ctau, p.settings.cutoff, p.settings.elastic_ratio)
    r = Ref{Ptr{Cvoid}}()
    check(ccall((:dp_physics_upload, lib), Cint,
                (Ptr{Cvoid}, Ref{DpSettings}, Cint, Cint, Ptr{Cdouble}, Ptr{Cvoid}, Ref{Ptr{Cvoid}}),
                ctx.h, st, length(p.tables), n, cols, C_NULL, r), ctx.h)
    GPUPhysics(ctx, r[])
end
# create_physics without Julia tables: PUMAS dE/dx files, or the portable table file
function create_physics_dedx(ctx::Context, files::Vector{String}, mats::Vector{DpMaterial};
                             settings = DpSettings(0.10565839, 658.654, 0.05, 0.05))
    r = Ref{Ptr{Cvoid}}()
    check(ccall((:dp_physics_create_dedx, lib), Cint,
                (Ptr{Cvoid}, Ref{DpSettings}, Cint, Ptr{DpMaterial}, Ptr{Cstring}, Ref{Ptr{Cvoid}}),
                ctx.h, settings, length(mats), mats, files, r), ctx.h)
    GPUPhysics(ctx, r[])
end
save_tables(g::GPUPhysics, path::AbstractString) =
    check(ccall((:dp_physics_save, lib), Cint, (Ptr{Cvoid}, Cstring), g.h, path), g.ctx.h)
function load_tables(ctx::Context, path::AbstractString)
    r = Ref{Ptr{Cvoid}}()
    check(ccall((:dp_physics_load, lib), Cint, (Ptr{Cvoid}, Cstring, Ref{Ptr{Cvoid}}),
                ctx.h, path, r), ctx.h)
    GPUPhysics(ctx, r[])
end

# ---------------------------------------------------------------- run_backward_mc
# src/Geometry.jl:1286-1338; precision 1 runs the FP32 transport and the FP32
# CSDA walk (within ~1e-6 of FP64 per history), 0 the reference's FP64 operations
function run_backward_mc(g::GPUPhysics; rock_thickness = 100.0, rock_density = 2650.0,
        elevation = 45.0, energy_min = 1.0, energy_max = nothing, n_samples = 10_000,
        compute_gradient = false, seed = 42, straggling = true, scattering = true,
        energy_threshold_low = 100.0, source_energy_max = nothing, primary_altitude = 3e4,
        precision = 0)
    p = DpMcParams(rock_thickness, rock_density, elevation, energy_min,
                   something(energy_max, energy_min), n_samples, UInt64(seed), straggling,
                   scattering, compute_gradient, energy_threshold_low,
                   something(source_energy_max, 0.0), primary_altitude, -1, -1, precision, -1,
                   0.0, 0.0)
    out = Ref{DpMcResult}()
    check(ccall((:dp_backward_mc, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpMcParams}, Ref{DpMcResult}),
                g.ctx.h, g.h, p, out), g.ctx.h)
    o = out[]
    (flux = o.flux, sigma = o.sigma,
     gradient = compute_gradient ? o.gradient : nothing,
     gradient_flux = compute_gradient ? o.gradient_flux : nothing,
     gradient_method = compute_gradient ? :deterministic_csda_sample_average : nothing,
     source_energy_max = o.source_energy_max)
end

# compute_flux (src/Geometry.jl:899) with the shallow porous layer: a layer
# routes the column through the stochastic kernels (CSDA steps when
# straggling = scattering = false)
function compute_flux(g::GPUPhysics, ρ, thickness, elevation, emin, emax; n_samples = 1000,
        seed = 42, straggling = true, scattering = true, energy_threshold_low = 100.0,
        porous_material = -1, porous_density = 0.0, porous_thickness = 0.0,
        primary_altitude = 3e4, precision = 0)
    p = DpMcParams(thickness, ρ, elevation, emin, emax, n_samples, UInt64(seed), straggling,
                   scattering, 0, energy_threshold_low, 0.0, primary_altitude, -1, -1, precision,
                   porous_material > 0 ? porous_material - 1 : -1, porous_density,
                   porous_thickness)
    out = Ref{DpMcResult}()
    check(ccall((:dp_backward_mc, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpMcParams}, Ref{DpMcResult}),
                g.ctx.h, g.h, p, out), g.ctx.h)
    out[].flux, out[].sigma
end

# compute_flux_differentiable with its rrule (src/Geometry.jl:958, :1007)
function flux_and_derivative(g::GPUPhysics, ρ, thickness, elevation, E, q; precision = 0)
    p = DpMcParams(thickness, ρ, elevation, 1.0, 1.0, 1, 0, 0, 0, 1, 100.0, 0.0, 3e4, -1, -1,
                   precision, -1, 0.0, 0.0)
    c = zeros(1); d = zeros(1)
    check(ccall((:dp_csda_flux_samples, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpMcParams}, Clong, Ptr{Cdouble}, Ptr{Cdouble},
                 Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Int32}),
                g.ctx.h, g.h, p, 1, [Float64(E)], [Float64(q)], [1.0], c, d, C_NULL), g.ctx.h)
    c[1], d[1]
end
compute_flux_differentiable(g::GPUPhysics, ρ, t, el, E, q) =
    first(flux_and_derivative(g, ρ, t, el, E, q))
function ChainRulesCore.rrule(::typeof(compute_flux_differentiable), g::GPUPhysics, ρ, t, el, E, q)
    f, dfdρ = flux_and_derivative(g, ρ, t, el, E, q)
    f, Δ -> (NoTangent(), NoTangent(), Δ * dfdρ, NoTangent(), NoTangent(), NoTangent(), NoTangent())
end

# ---------------------------------------------------------------- mixtures, batches
# runtime mixtures with their MIXED kernels (MaterialMixture, prepare_mixed_kernel)
mutable struct GPUMixture; h::Ptr{Cvoid}; end
function GPUMixture(g::GPUPhysics, m::DiffPumas.MaterialMixture)
    mats = Cint.(m.materials .- 1); fr = Float64.(m.fractions)
    r = Ref{Ptr{Cvoid}}()
    check(ccall((:dp_mixture_prepare, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Cint}, Ptr{Cdouble}, Ref{Ptr{Cvoid}}),
                g.ctx.h, g.h, length(mats), mats, fr, r), g.ctx.h)
    x = GPUMixture(r[])
    finalizer(x -> ccall((:dp_mixture_free, lib), Cint, (Ptr{Cvoid},), x.h), x)
end
GPUMixture(g::GPUPhysics, material::Int) = GPUMixture(g, DiffPumas.MaterialMixture(material))

# many run_backward_mc estimates in one launch (one per line of sight)
function run_backward_mc_batch(g::GPUPhysics, rock::GPUMixture, air::GPUMixture,
                               los::Vector{DpLos}; seed = 42, straggling = true,
                               scattering = true, energy_threshold_low = 100.0, precision = 1,
                               compute_gradient = false)
    cfg = DpMcConfig(straggling, scattering, energy_threshold_low, 0.0, UInt64(seed), precision)
    out = Vector{DpLosResult}(undef, length(los))
    check(ccall((:dp_mc_los, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpMcConfig}, Clong,
                 Ptr{DpLos}, Cint, Ptr{DpLosResult}),
                g.ctx.h, g.h, rock.h, air.h, cfg, length(los), los, compute_gradient, out), g.ctx.h)
    out
end
# with the shallow porous layer of each line (its porous_thickness / porous_density)
function run_backward_mc_batch(g::GPUPhysics, rock::GPUMixture, porous::GPUMixture,
                               air::GPUMixture, los::Vector{DpLos}; seed = 42,
                               straggling = true, scattering = true,
                               energy_threshold_low = 100.0, precision = 1)
    cfg = DpMcConfig(straggling, scattering, energy_threshold_low, 0.0, UInt64(seed), precision)
    out = Vector{DpLosResult}(undef, length(los))
    check(ccall((:dp_mc_los_layers, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpMcConfig},
                 Clong, Ptr{DpLos}, Cint, Ptr{DpLosResult}),
                g.ctx.h, g.h, rock.h, porous.h, air.h, cfg, length(los), los, 0, out), g.ctx.h)
    out
end

# compute_directional_flux_mc (src/Tomography.jl:979) for many paths at once
function directional_flux_mc(g::GPUPhysics, matcfg, site, paths::Vector{DirectionalPath},
                             cell_materials, cell_densities, samples::Vector{EnergySample},
                             seed::Int; straggling = true, energy_threshold_low = 100.0,
                             precision = 1)
    # media set: rock, the distinct cell mixtures, air (leading media are staged on chip)
    uniq = unique(cell_materials)
    media = [GPUMixture(g, matcfg.rock_material); [GPUMixture(g, m) for m in uniq];
             GPUMixture(g, matcfg.air_material)]
    idx = Dict(m => k for (k, m) in enumerate(uniq))          # 0-based: rock is 0
    set = Ref{Ptr{Cvoid}}()
    check(ccall((:dp_dir_media_create, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Ptr{Ptr{Cvoid}}, Ref{Ptr{Cvoid}}),
                g.ctx.h, g.h, length(media), [m.h for m in media], set), g.ctx.h)
    cosθ = [cosd(p.zenith) for p in paths]
    segs = [p.valid ? p.segments : CellSegment[] for p in paths]
    seg_ptr = Int64[0; cumsum(length.(segs))]
    seg_medium = Int32[idx[cell_materials[s.cell_idx]] for ss in segs for s in ss]
    seg_density = Float64[cell_densities[s.cell_idx] for ss in segs for s in ss]
    seg_length = Float64[s.distance for ss in segs for s in ss]
    n = length(samples)
    sample_ptr = Int64.(0:n:n * length(paths))                # the same samples per path
    E = repeat([s.energy for s in samples], length(paths))
    q = repeat([s.charge for s in samples], length(paths))
    w = repeat([s.weight for s in samples], length(paths))
    rem = [p.remaining_rock_distance for p in paths]
    air = [max(0.0, site.primary_altitude - p.surface_exit_z) / max(c, 1e-3)
           for (p, c) in zip(paths, cosθ)]
    valid = Int32[p.valid && c > 0 for (p, c) in zip(paths, cosθ)]
    out = Vector{DpLosResult}(undef, length(paths))
    GC.@preserve cosθ rem air valid seg_ptr seg_medium seg_density seg_length sample_ptr E q w begin
        b = DpDirBatch(length(paths), pointer(cosθ), pointer(rem), pointer(air), pointer(valid),
                       pointer(seg_ptr), pointer(seg_medium), pointer(seg_density),
                       pointer(seg_length), pointer(sample_ptr), pointer(E), pointer(q),
                       pointer(w), 0.0, 0.0, 0, length(media) - 1, matcfg.rock_density,
                       site.detector_elevation)
        cfg = DpMcConfig(straggling, false, energy_threshold_low, 0.0, UInt64(seed), precision)
        rc = ccall((:dp_dir_mc, lib), Cint,
                   (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpDirBatch}, Ref{DpMcConfig},
                    Ptr{DpLosResult}, Ptr{Cdouble}, Ptr{Int32}, Ptr{Cdouble}),
                   g.ctx.h, g.h, set[], b, cfg, out, C_NULL, C_NULL, C_NULL)
        ccall((:dp_dir_media_free, lib), Cint, (Ptr{Cvoid},), set[])
        check(rc, g.ctx.h)
    end
    [(o.flux, o.sigma) for o in out]
end

# ---------------------------------------------------------------- water-fraction operator
# make_csda_operator (src/Tomography.jl): the flux of every bin and its sparse
# Jacobian in water fraction from one dp_dir_csda launch
function make_csda_operator(g::GPUPhysics, shallow, matcfg, site, paths, samples; n_cells,
                            valid_bins, precision = 0)
    sub = paths[valid_bins]
    seg_ptr = Int64[0; cumsum(length.(getfield.(sub, :segments)))]
    cells = Int32[s.cell_idx - 1 for p in sub for s in p.segments]
    lens = Float64[s.distance for p in sub for s in p.segments]
    rows = reduce(vcat, [fill(b, length(p.segments)) for (b, p) in enumerate(sub)]; init = Int[])
    c, mc = get_csda_correction(), get_csda_material_correction()
    cfg = DpCsdaConfig(matcfg.rock_material - 1, matcfg.water_material - 1,
                       matcfg.air_material - 1,
                       matcfg.porous_material > 0 ? matcfg.porous_material - 1 : -1,
                       matcfg.rock_density, matcfg.water_density, matcfg.porous_density,
                       matcfg.porous_top_thickness, site.detector_elevation, site.primary_altitude,
                       c.enabled, c.kappa_strag, c.kappa_hard, c.resid_a, c.resid_b, c.resid_c,
                       c.resid_d, mc.enabled, mc.linear, mc.quadratic)
    cosθ = [cosd(p.zenith) for p in sub]; rem = [p.remaining_rock_distance for p in sub]
    ez = [p.surface_exit_z for p in sub]; valid = Int32.(getfield.(sub, :valid))
    E = [s.energy for s in samples]; q = [s.charge for s in samples]
    wt = [s.weight for s in samples]
    sh = UInt8.(shallow)
    return function (w)
        flux = zeros(length(sub)); jac = zeros(length(cells))
        GC.@preserve cosθ rem ez valid seg_ptr cells lens E q wt begin
            b = DpCsdaBatch(length(sub), pointer(cosθ), pointer(rem), pointer(ez), pointer(valid),
                            pointer(seg_ptr), pointer(cells), pointer(lens), length(E), pointer(E),
                            pointer(q), pointer(wt))
            check(ccall((:dp_dir_csda, lib), Cint,
                        (Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpCsdaConfig}, Ref{DpCsdaBatch}, Clong,
                         Ptr{UInt8}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cint),
                        g.ctx.h, g.h, cfg, b, n_cells, sh, w, flux, jac, precision), g.ctx.h)
        end
        flux, sparse(rows, cells .+ 1, jac, length(sub), n_cells)   # sparse() sums repeats
    end
end

# ---------------------------------------------------------------- voxel tomography
# trace once (precompute_paths), evaluate often
mutable struct Paths; h::Ptr{Cvoid}; ctx::Context; n_rays::Int; ncell::Int; end
function Paths(ctx::Context, grid::DpGrid, rays::Vector{DpRay}; side_cell = -1)
    r = Ref{Ptr{Cvoid}}()
    check(ccall((:dp_tomo_paths_create, lib), Cint,
                (Ptr{Cvoid}, Ref{DpGrid}, Clong, Ptr{DpRay}, Cint, Ref{Ptr{Cvoid}}),
                ctx.h, grid, length(rays), rays, side_cell, r), ctx.h)
    p = Paths(r[], ctx, length(rays), grid.nx * grid.ny * grid.nz)
    finalizer(p -> ccall((:dp_tomo_paths_free, lib), Cint, (Ptr{Cvoid},), p.h), p)
end
# flux per ray and J^T r (deterministic, no atomics); tp's node arrays are host
# pointers (pointer(x) under GC.@preserve x)
function flux_and_vjp(g::GPUPhysics, P::Paths, tp::DpTomoParams, ρ::Vector{Float64},
                      r::Vector{Float64})
    flux = zeros(P.n_rays); grad = zeros(P.ncell)
    check(ccall((:dp_tomo_eval, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpTomoParams}, Ptr{Cdouble}, Ptr{Cdouble},
                 Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                g.ctx.h, g.h, P.h, tp, ρ, r, flux, grad, C_NULL), g.ctx.h)
    flux, grad
end
tomo_flux(g::GPUPhysics, P::Paths, tp::DpTomoParams, ρ) = first(flux_and_vjp(g, P, tp, ρ, zeros(P.n_rays)))
# the forward operator with its rrule, for make_csda_operator-style solvers
function ChainRulesCore.rrule(::typeof(tomo_flux), g::GPUPhysics, P::Paths, tp::DpTomoParams, ρ)
    flux = tomo_flux(g, P, tp, ρ)
    flux, Δ -> (NoTangent(), NoTangent(), NoTangent(), NoTangent(),
                last(flux_and_vjp(g, P, tp, ρ, collect(Float64, Δ))))
end

# the inversion loops on the device (src/Tomography_inverse.jl): SART (0),
# Gauss-Newton (1), MLEM (2), gradient descent (3); obs, w, ρ and hist are
# device pointers (CUDA.jl: pointer(cu_array)), ρ is updated in place
solve!(g::GPUPhysics, P::Paths, tp::DpTomoParams, obs::Ptr{Cdouble}, w::Ptr{Cdouble},
       ρ::Ptr{Cdouble}, sp::DpSolveParams, hist::Vector{Float64}) =
    check(ccall((:dp_tomo_solve_dev, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpTomoParams}, Ptr{Cdouble},
                 Ptr{Cdouble}, Ptr{Cdouble}, Ref{DpSolveParams}, Ptr{Cdouble}),
                g.ctx.h, g.h, P.h, tp, obs, w, ρ, sp, hist), g.ctx.h)

# flux and J^T r without any device allocation inside the call (mixed
# precision, a fixed scratch inside the library): for hosts whose device
# memory is owned by a pool allocator; device pointers
eval_noalloc!(g::GPUPhysics, P::Paths, tp::DpTomoParams, ρ::Ptr{Cdouble}, cot::Ptr{Cdouble},
              flux::Ptr{Cdouble}, grad::Ptr{Cdouble}) =
    check(ccall((:dp_tomo_eval_noalloc_dev, lib), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpTomoParams}, Ptr{Cdouble},
                 Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                g.ctx.h, g.h, P.h, tp, ρ, cot, flux, grad), g.ctx.h)

# ---------------------------------------------------------------- launch shapes
# the workload is a C callback (@cfunction) that runs the caller's batch
const TUNE_WORK = Ref{Any}()
run_cb(::Ptr{Cvoid})::Cint = (TUNE_WORK[](); Cint(0))
function autotune!(g::GPUPhysics, family::Integer, precision::Integer, work)
    TUNE_WORK[] = work
    best = Ref{DpMcShape}(DpMcShape(0, 0, 0, 0))
    tried = Vector{DpMcShape}(undef, 16); ms = zeros(16); n = Ref{Cint}(0)
    check(ccall((:dp_autotune_shape, lib), Cint,
                (Ptr{Cvoid}, Cint, Cint, Ptr{Cvoid}, Ptr{Cvoid}, Ref{DpMcShape}, Ptr{DpMcShape},
                 Ptr{Cdouble}, Cint, Ref{Cint}),
                g.ctx.h, family, precision, @cfunction(run_cb, Cint, (Ptr{Cvoid},)), C_NULL,
                best, tried, ms, 16, n), g.ctx.h)
    best[], collect(zip(tried[1:min(n[], 16)], ms[1:min(n[], 16)]))
end
set_shape!(g::GPUPhysics, family::Integer, precision::Integer, s::DpMcShape) =
    check(ccall((:dp_set_mc_shape, lib), Cint, (Ptr{Cvoid}, Cint, Cint, Ref{DpMcShape}),
                g.ctx.h, family, precision, s), g.ctx.h)

# ---------------------------------------------------------------- terrain, meshes
# mesh.pointlist (3 x n) and mesh.tetrahedronlist (4 x m, one-based) map directly
function tetra_neighbors(m::DpTetraMesh)
    nb = zeros(Int32, 4, m.n_tets)
    ccall((:dp_tetra_neighbors, lib), Cint, (Ref{DpTetraMesh}, Ptr{Int32}), m, nb) == 0 ||
        throw(ArgumentError("invalid tetrahedral mesh"))
    nb
end
# ray_surface_exit_distance for many directions
function surface_exit(t::DpTerrain, zenith::Vector{Float64}, azimuth::Vector{Float64})
    n = length(zenith)
    d = zeros(n); z = zeros(n); ok = zeros(Int32, n)
    ccall((:dp_surface_exit, lib), Cint,
          (Ref{DpTerrain}, Clong, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Int32}),
          t, n, zenith, azimuth, d, z, ok) == 0 || throw(ArgumentError("invalid terrain"))
    d, z, ok .!= 0
end

end # module
