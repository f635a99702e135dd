"""
    PorousMaterialsGB300

`ccall` binding of libpmgb (the sm_103a Widom-insertion / energy-grid library, C ABI in
include/pmgb.h) for PorousMaterials.jl v0.4.  It provides drop-in bodies for

  * `henry_coefficient(crystal, molecule, temperature, ljff; insertions_per_volume,
     verbose, ewald_precision, autosave, filename_comment, accessibility_grid)`
                                                                 (src/henry.jl:34-181)
  * `energy_grid(crystal, molecule, ljff; resolution, n_rotations, temperature, units,
     center, verbose)`                                           (src/grid.jl:291-362)

plus the derivative of K_H with respect to the pure-species LJ parameters and the framework
charge scale (a ChainRulesCore `rrule`), and batched screening of many frameworks in one
launch.  Everything before and after the insertion loop (replication, Ewald set-up, block
statistics, the result `Dict`, autosave) is the reference's own code path, called unchanged.

Set `ENV["PMGB_LIB"]` to the built `libpmgb.so` before loading the module.
"""
module PorousMaterialsGB300

using PorousMaterials
using JLD2
using Printf
using Statistics
import ChainRulesCore

const LIB = get(ENV, "PMGB_LIB", joinpath(@__DIR__, "..", "pmgb", "libpmgb.so"))
const N_BLOCKS = 5  # src/mc_helpers.jl:11

# ---------------------------------------------------------------------------- context
mutable struct Context
    ptr::Ptr{Cvoid}
    function Context(device::Integer=0)
        out = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:pmgb_create, LIB), Cint, (Cint, Ptr{Ptr{Cvoid}}), device, out)
        rc == 0 || error("libpmgb: ", unsafe_string(ccall((:pmgb_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL)))
        ctx = new(out[])
        finalizer(c -> ccall((:pmgb_destroy, LIB), Cvoid, (Ptr{Cvoid},), c.ptr), ctx)
        return ctx
    end
end

const DEFAULT_CONTEXT = Ref{Union{Nothing, Context}}(nothing)
function default_context()
    if DEFAULT_CONTEXT[] === nothing
        DEFAULT_CONTEXT[] = Context(0)
    end
    return DEFAULT_CONTEXT[]
end

function check(ctx::Context, rc::Integer)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:pmgb_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx.ptr))
    error("libpmgb ($rc): $msg")
end

# ---------------------------------------------------------------------------- systems
"""
A replicated crystal + guest + force field resident on the GPU (pmgb_system_create).
`species` orders the ε / σ² tables; `charge_scale` scales every framework charge.
"""
mutable struct GPUSystem
    ptr::Ptr{Cvoid}
    ctx::Context
    species::Vector{Symbol}
    charged::Bool
    function GPUSystem(ctx::Context, crystal::Crystal, molecule::Molecule, ljff::LJForceField;
                       eparams::Union{Nothing, PorousMaterials.EwaldParams}=nothing, charge_scale::Float64=1.0,
                       pure_ϵ::Union{Nothing, Dict{Symbol, Float64}}=nothing,
                       pure_σ::Union{Nothing, Dict{Symbol, Float64}}=nothing, refine_tail::Float64=0.0)
        species = unique(vcat(crystal.atoms.species, molecule.atoms.species))
        sid = Dict(s => Int32(i - 1) for (i, s) in enumerate(species))
        n = length(species)
        ϵ = Matrix{Float64}(undef, n, n)
        σ² = Matrix{Float64}(undef, n, n)
        for (j, b) in enumerate(species), (i, a) in enumerate(species)
            if isnothing(pure_ϵ)
                ϵ[i, j] = ljff.ϵ[a][b]
                σ²[i, j] = ljff.σ²[a][b]
            else  # Lorentz-Berthelot from (perturbed) pure parameters, src/forcefield.jl:97-108
                ϵ[i, j] = sqrt(pure_ϵ[a] * pure_ϵ[b])
                σ²[i, j] = ((pure_σ[a] + pure_σ[b]) / 2)^2
            end
        end
        mcart = Cart(molecule, crystal.box)
        gx = mcart.atoms.coords.x .- mcart.com.x     # offsets from the centre of mass (3 x n)
        qx = mcart.charges.coords.x .- mcart.com.x
        out = Ref{Ptr{Cvoid}}(C_NULL)
        check(ctx, ccall((:pmgb_system_create, LIB), Cint,
            (Ptr{Cvoid}, Ptr{Float64}, Int32, Ptr{Float64}, Ptr{Int32}, Int32, Ptr{Float64}, Ptr{Float64},
             Int32, Ptr{Float64}, Ptr{Float64}, Float64, Int32, Ptr{Float64}, Ptr{Int32}, Int32,
             Ptr{Float64}, Ptr{Float64}, Ptr{Ptr{Cvoid}}),
            ctx.ptr, Matrix{Float64}(crystal.box.f_to_c), crystal.atoms.n, Matrix{Float64}(crystal.atoms.coords.xf),
            Int32[sid[s] for s in crystal.atoms.species], crystal.charges.n,
            Matrix{Float64}(crystal.charges.coords.xf), crystal.charges.q .* charge_scale,
            n, ϵ, σ², ljff.r²_cutoff, molecule.atoms.n, Matrix{Float64}(gx),
            Int32[sid[s] for s in molecule.atoms.species], molecule.charges.n, Matrix{Float64}(qx),
            Vector{Float64}(molecule.charges.q), out))
        sys = new(out[], ctx, species, has_charges(crystal) && has_charges(molecule))
        finalizer(s -> ccall((:pmgb_system_destroy, LIB), Cvoid, (Ptr{Cvoid},), s.ptr), sys)
        if sys.charged
            isnothing(eparams) && error("a charged system needs Ewald parameters")
            kabc = Int32[v for k in eparams.kvecs for v in (k.ka, k.kb, k.kc)]
            wt = Float64[k.wt for k in eparams.kvecs]
            check(ctx, ccall((:pmgb_system_set_ewald, LIB), Cint,
                (Ptr{Cvoid}, Float64, Float64, Int32, Ptr{Int32}, Ptr{Float64}),
                sys.ptr, eparams.α, eparams.sr_cutoff_r, length(wt), kabc, wt))
        end
        if refine_tail > 0  # FP64-grade re-evaluation of the Boltzmann tail: K_H within 1e-6
            check(ctx, ccall((:pmgb_system_set_refine, LIB), Cint, (Ptr{Cvoid}, Float64), sys.ptr, refine_tail))
        end
        return sys
    end
end

"""
    widom_blocks(sys, nb_per_block, temperature; seed) -> 4 x N_BLOCKS

Replaces the pmap over blocks of _conduct_Widom_insertions (src/henry.jl:103-113):
column b = (log Σ e^{-U/T}, ⟨U_vdw⟩, ⟨U_es⟩, #insertions with U = Inf).
"""
function widom_blocks(sys::GPUSystem, nb_per_block::Integer, temperature::Float64; seed::UInt64=rand(UInt64))
    out = zeros(4, N_BLOCKS)
    check(sys.ctx, ccall((:pmgb_widom, LIB), Cint,
        (Ptr{Cvoid}, Int64, Int32, UInt64, Float64, Ptr{Float64}, Ptr{Float64}),
        sys.ptr, nb_per_block, N_BLOCKS, seed, temperature, out, C_NULL))
    return out
end

"""
    widom_adjoint(sys, nb_per_block, temperature; seed) -> (blocks, dθ)

pmgb_widom_adjoint: block results plus Σ w ∂U/∂θ; see include/pmgb.h for the layout of dθ.
"""
function widom_adjoint(sys::GPUSystem, nb_per_block::Integer, temperature::Float64; seed::UInt64=rand(UInt64))
    n = length(sys.species)
    blocks = zeros(4, N_BLOCKS)
    dθ = zeros(3 + 2 * n * n)
    check(sys.ctx, ccall((:pmgb_widom_adjoint, LIB), Cint,
        (Ptr{Cvoid}, Int64, Int32, UInt64, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float32}),
        sys.ptr, nb_per_block, N_BLOCKS, seed, temperature, blocks, dθ, C_NULL, C_NULL))
    return blocks, dθ
end

"""
    set_centre_image!(sys, on); centre_image(sys) -> Bool

pmgb_system_set_centre_image / pmgb_system_centre_image: Widom distances from the pose centre
for guests with several sites, where every width of the supercell is at least
2 (cutoff + guest reach) + 0.1 Å (on by default; the per-site form differs by FP32 rounding only).
"""
set_centre_image!(sys::GPUSystem, on::Bool) =
    check(sys.ctx, ccall((:pmgb_system_set_centre_image, LIB), Cint, (Ptr{Cvoid}, Int32), sys.ptr, Int32(on)))

function centre_image(sys::GPUSystem)
    on = Ref{Int32}(0)
    check(sys.ctx, ccall((:pmgb_system_centre_image, LIB), Cint, (Ptr{Cvoid}, Ptr{Int32}), sys.ptr, on))
    return on[] != 0
end

# ---------------------------------------------------------------------------- drop-in bodies
"""
Drop-in for `henry_coefficient` (src/henry.jl:34-181): the same arguments and keywords, the same
block statistics, result keys, units and autosave file; the insertions run on the GPU.
`accessibility_grid` (a `Grid{Bool}` over the unit cell) gates the insertions as in the reference:
an insertion whose nearest grid node and its 26 neighbours are all inaccessible gets U = Inf.
`seed` makes a run reproducible; `refine_tail` (default 1e-3) re-evaluates in high precision the
insertions that carry all but that fraction of each block's Boltzmann weight, which keeps K_H
within 1e-6 of an FP64 evaluation.
"""
function henry_coefficient(crystal::Crystal, molecule::Molecule, temperature::Float64,
                           ljforcefield::LJForceField; insertions_per_volume::Union{Int, Float64}=200,
                           verbose::Bool=true, ewald_precision::Float64=1e-6, autosave::Bool=true,
                           filename_comment::AbstractString="",
                           accessibility_grid::Union{Nothing, Grid{Bool}}=nothing,
                           seed::UInt64=rand(UInt64), ctx::Context=default_context(), refine_tail::Float64=1e-3)
    assert_P1_symmetry(crystal)
    # the grid must describe this crystal's unit cell (the reference checks this under `verbose`;
    # a mismatched grid would gate the wrong pockets, so it is checked on every call here)
    if !isnothing(accessibility_grid) && !isapprox(accessibility_grid.box, crystal.box)
        error(@sprintf("accessibility grid box does not match box of %s.\n", crystal.name))
    end
    t0 = time()
    n_total = max(N_BLOCKS, ceil(Int, insertions_per_volume * crystal.box.Ω))   # before replication
    n_per_block = ceil(Int, n_total / N_BLOCKS)
    repfactors = replication_factors(crystal.box, ljforcefield)
    supercell = replicate(crystal, repfactors)
    guest = Frac(molecule, supercell.box)
    charged = has_charges(supercell) && has_charges(guest)
    ρ = crystal_density(supercell)
    ep = charged ? setup_Ewald_sum(supercell.box, sqrt(ljforcefield.r²_cutoff); ϵ=ewald_precision,
                                   verbose=verbose) : nothing
    sys = GPUSystem(ctx, supercell, guest, ljforcefield; eparams=ep, refine_tail=refine_tail)
    if !isnothing(accessibility_grid)
        verbose && println("Using provided accessibility grid to block inaccessible pockets")
        set_accessibility!(sys, accessibility_grid, repfactors)
    end
    blocks = widom_blocks(sys, n_per_block, temperature; seed=seed)

    # per block: K_H = Σ e^{-U/T} / (R T n), ⟨U⟩ weighted by e^{-U/T}; errors 2σ/√N_BLOCKS
    R = PorousMaterials.UNIV_GAS_CONST
    kh = exp.(blocks[1, :] .- log(R * temperature * n_per_block))
    u_vdw = blocks[2, :]
    u_es = charged ? blocks[3, :] : zeros(N_BLOCKS)
    two_se(v) = 2.0 * std(v) / sqrt(N_BLOCKS)
    kj = PorousMaterials.K_TO_KJ_PER_MOL
    kh_molar = mean(kh)
    kh_mass = kh_molar / ρ
    uv, ue = mean(u_vdw), mean(u_es)
    results = Dict{String, Any}(
        "xtal" => supercell.name,
        "henry coefficient [mol/(m³-bar)]" => kh_molar,
        "henry coefficient [mmol/(g-bar)]" => kh_mass,
        "err henry coefficient [mmol/(g-bar)]" => two_se(kh) / ρ,
        "henry coefficient [mol/(kg-Pa)]" => kh_mass / 100000.0,
        "⟨U, vdw⟩ (K)" => uv,
        "⟨U, es⟩ (K)" => ue,
        "⟨U⟩ (K)" => uv + ue,
        "⟨U⟩ (kJ/mol)" => (uv + ue) * kj,
        "⟨U, vdw⟩ (kJ/mol)" => uv * kj,
        "err ⟨U, vdw⟩ (kJ/mol)" => two_se(u_vdw) * kj,
        "⟨U, es⟩ (kJ/mol)" => ue * kj,
        "err ⟨U, es⟩ (kJ/mol)" => two_se(u_es) * kj,
        "Qst (kJ/mol)" => -(uv + ue) * kj + temperature * kj,
        "err Qst (kJ/mol)" => (two_se(u_vdw) + two_se(u_es)) * kj,
        "elapsed time (min)" => (time() - t0) / 60)
    if autosave
        dir = rc[:paths][:simulations]
        isdir(dir) || mkdir(dir)
        file = joinpath(dir, henry_result_savename(supercell, molecule, temperature, ljforcefield,
                                                   insertions_per_volume, comment=filename_comment))
        @save file results
        verbose && println("\tResults saved in: ", file)
    end
    if verbose
        for (name, v, err) in (("henry coefficient [mmol/(g-bar)]", kh_mass, two_se(kh) / ρ),
                               ("⟨U, vdw⟩ (kJ/mol)", uv * kj, two_se(u_vdw) * kj),
                               ("⟨U, es⟩ (kJ/mol)", ue * kj, two_se(u_es) * kj),
                               ("Qst (kJ/mol)", results["Qst (kJ/mol)"], results["err Qst (kJ/mol)"]))
            @printf("\t%s = %f +/- %f\n", name, v, err)
        end
    end
    return results
end

"""
    set_accessibility!(sys, grid, repfactors)

pmgb_system_set_accessibility: gate this system's Widom insertions by a `Grid{Bool}` over the unit
cell (src/henry.jl:225 -> accessible, src/grid.jl:778-836); `repfactors` is the replication of the
system's supercell.
"""
function set_accessibility!(sys::GPUSystem, grid::Grid{Bool}, repfactors)
    data = UInt8.(grid.data)        # column-major, i fastest: the ABI's layout
    check(sys.ctx, ccall((:pmgb_system_set_accessibility, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{UInt8}),
        sys.ptr, Int32[size(data)...], Int32[repfactors...], data))
end

"""
Drop-in for `energy_grid` (src/grid.jl:291-362): the same arguments and keywords.  A single-site
probe gets its van der Waals energy at every point (pmgb_energy_grid, exact to the FP64 tolerance).
A probe with several sites (or charges) gets the Boltzmann-weighted rotational average
-T log(⟨e^{-U/T}⟩) over `n_rotations` uniform random orientations at `temperature`
(pmgb_energy_grid_rotational), with the electrostatic energy included where both the crystal and the
probe are charged, as the reference's rotational branch defines it.
"""
function energy_grid(crystal::Crystal, molecule::Molecule{Cart}, ljforcefield::LJForceField;
                     resolution::Union{Float64, Tuple{Int, Int, Int}}=1.0, n_rotations::Int=1000,
                     temperature::Float64=NaN, units::Symbol=:kJ_mol, center::Bool=false,
                     verbose::Bool=true, seed::UInt64=rand(UInt64), ctx::Context=default_context())
    assert_P1_symmetry(crystal)
    units in (:kJ_mol, :K) || error("Pass :kJ_mol or :K for units of kJ/mol or K, respectively.")
    rotations = needs_rotations(molecule)
    if rotations && isnan(temperature)
        error("Must pass temperature (K) for Boltzmann weighted rotations.\n")
    end
    n_pts = isa(resolution, Tuple{Int, Int, Int}) ? resolution : required_n_pts(crystal.box, resolution)
    repfactors = replication_factors(crystal.box, ljforcefield)
    supercell = replicate(crystal, repfactors)
    guest = Frac(molecule, supercell.box)
    factor = units == :kJ_mol ? 8.314 / 1000.0 : 1.0     # the factor src/grid.jl:357-359 applies
    data = Array{Float32}(undef, n_pts...)                # column-major: i fastest, as the ABI writes
    if rotations
        charged = has_charges(supercell) && has_charges(guest)
        ep = charged ? setup_Ewald_sum(supercell.box, sqrt(ljforcefield.r²_cutoff); verbose=verbose) : nothing
        sys = GPUSystem(ctx, supercell, guest, ljforcefield; eparams=ep)
        check(ctx, ccall((:pmgb_energy_grid_rotational, LIB), Cint,
            (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Int32, Float64, UInt64, Float64, Ptr{Float32}),
            sys.ptr, Int32[n_pts...], Int32[repfactors...], n_rotations, temperature, seed, factor, data))
    else
        sys = GPUSystem(ctx, supercell, guest, ljforcefield)
        check(ctx, ccall((:pmgb_energy_grid, LIB), Cint,
            (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Float64, Ptr{Float32}),
            sys.ptr, Int32[n_pts...], Int32[repfactors...], factor, data))
    end
    return Grid(crystal.box, n_pts, Float64.(data), units,
                center ? crystal.box.f_to_c * [-0.5, -0.5, -0.5] : [0.0, 0.0, 0.0])
end

# ---------------------------------------------------------------------------- derivatives
"""
    henry_kh(crystal, molecule, temperature, ljff, ϵ, σ, λ; insertions_per_volume, seed)

Block-mean K_H (mol/(m³ bar)) as a function of the pure-species parameters `ϵ`, `σ`
(vectors over `species(ljff, crystal, molecule)`) and the framework charge scale `λ`, with
Lorentz-Berthelot mixing.  Differentiable through the `rrule` below (pmgb_widom_adjoint:
pair terms recomputed, no tape).
"""
species_of(crystal, molecule) = unique(vcat(crystal.atoms.species, molecule.atoms.species))

function _setup(crystal, molecule, ljff, insertions_per_volume, ewald_precision)
    nb = ceil(Int, max(N_BLOCKS, ceil(Int, insertions_per_volume * crystal.box.Ω)) / N_BLOCKS)
    sc = replicate(crystal, replication_factors(crystal.box, ljff))
    mol = Frac(molecule, sc.box)
    charged = has_charges(sc) && has_charges(mol)
    ep = charged ? setup_Ewald_sum(sc.box, sqrt(ljff.r²_cutoff); ϵ=ewald_precision) : nothing
    return sc, mol, ep, nb
end

function henry_kh(crystal, molecule, temperature, ljff, ϵ::AbstractVector, σ::AbstractVector, λ::Real;
                  insertions_per_volume=200, ewald_precision=1e-6, seed::UInt64=UInt64(1),
                  ctx::Context=default_context())
    sp = species_of(crystal, molecule)
    sc, mol, ep, nb = _setup(crystal, molecule, ljff, insertions_per_volume, ewald_precision)
    sys = GPUSystem(ctx, sc, mol, ljff; eparams=ep, charge_scale=Float64(λ),
                    pure_ϵ=Dict(zip(sp, ϵ)), pure_σ=Dict(zip(sp, σ)))
    blocks = widom_blocks(sys, nb, temperature; seed=seed)
    return mean(exp.(blocks[1, :] .- log(PorousMaterials.UNIV_GAS_CONST * temperature * nb)))
end

function ChainRulesCore.rrule(::typeof(henry_kh), crystal, molecule, temperature, ljff,
                              ϵ::AbstractVector, σ::AbstractVector, λ::Real; insertions_per_volume=200,
                              ewald_precision=1e-6, seed::UInt64=UInt64(1), ctx::Context=default_context())
    sp = species_of(crystal, molecule)
    n = length(sp)
    sc, mol, ep, nb = _setup(crystal, molecule, ljff, insertions_per_volume, ewald_precision)
    sys = GPUSystem(ctx, sc, mol, ljff; eparams=ep, charge_scale=Float64(λ),
                    pure_ϵ=Dict(zip(sp, ϵ)), pure_σ=Dict(zip(sp, σ)))
    blocks, dθ = widom_adjoint(sys, nb, temperature; seed=seed)
    R = PorousMaterials.UNIV_GAS_CONST
    kh = mean(exp.(blocks[1, :] .- log(R * temperature * nb)))
    scale = -exp(dθ[1]) / (temperature * R * temperature * nb * N_BLOCKS)
    # dθ[4 + 2((a-1) n + (b-1))]: Σ w ∂U/∂ε_ab; +1: Σ w ∂U/∂σ²_ab (a guest, b framework; 0-based in C)
    dϵ_ab = [dθ[4 + 2 * ((a - 1) * n + (b - 1))] * scale for a in 1:n, b in 1:n]
    dσ²_ab = [dθ[5 + 2 * ((a - 1) * n + (b - 1))] * scale for a in 1:n, b in 1:n]
    gϵ = zeros(n)
    gσ = zeros(n)
    for a in 1:n, b in 1:n
        ϵab = sqrt(ϵ[a] * ϵ[b])
        for s in (a == b ? (a,) : (a, b))
            gϵ[s] += dϵ_ab[a, b] * (a == b ? 1.0 : 0.5 * ϵab / ϵ[s])
            gσ[s] += dσ²_ab[a, b] * (a == b ? 2σ[a] : 0.5 * (σ[a] + σ[b]))
        end
    end
    gλ = sys.charged ? dθ[3] * scale / λ : 0.0   # U_es is linear in λ: ∂U_es/∂λ = U_es(λ) / λ
    function henry_kh_pullback(Δ)
        return (ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(),
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), Δ .* gϵ, Δ .* gσ, Δ * gλ)
    end
    return kh, henry_kh_pullback
end

# ---------------------------------------------------------------------------- batched screening
"""
    henry_screen(crystals, molecule, temperature, ljff; insertions=20_000, seed=0, tune=true,
                 return_energies=false)

K_H (mol/(m³ bar)) of every crystal from one persistent, graph-captured launch
(pmgb_batch_*).  System s uses the Philox key seed + s * 0x9E3779B97F4A7C15.  With
`return_energies`, also each crystal's per-insertion energies as a 2 x n matrix
(U_vdw, U_es in K; pmgb_batch_energies).
"""
function henry_screen(crystals::Vector{Crystal}, molecule::Molecule, temperature::Float64, ljff::LJForceField;
                      insertions::Int=20_000, seed::Integer=0, tune::Bool=true, ewald_precision=1e-6,
                      ctx::Context=default_context(), refine_tail::Float64=1e-3, return_energies::Bool=false)
    nb = cld(insertions, N_BLOCKS)
    systems = GPUSystem[]
    for cr in crystals
        sc, mol, ep, _ = _setup(cr, molecule, ljff, 0, ewald_precision)
        push!(systems, GPUSystem(ctx, sc, mol, ljff; eparams=ep))
    end
    handle = Ref{Ptr{Cvoid}}(C_NULL)
    check(ctx, ccall((:pmgb_batch_create, LIB), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Int64}, Int32, Int32, Ptr{Ptr{Cvoid}}),
        ctx.ptr, length(systems), [s.ptr for s in systems], fill(Int64(nb), length(systems)), N_BLOCKS, 0,
        handle))
    try
        refine_tail > 0 && check(ctx, ccall((:pmgb_batch_set_refine, LIB), Cint, (Ptr{Cvoid}, Float64),
                                            handle[], refine_tail))
        if tune
            best = Ref{Float64}(0.0)
            check(ctx, ccall((:pmgb_batch_tune, LIB), Cint, (Ptr{Cvoid}, UInt64, Float64, Int32, Ptr{Float64}),
                             handle[], UInt64(seed + 1), temperature, 3, best))
        end
        check(ctx, ccall((:pmgb_batch_launch, LIB), Cint, (Ptr{Cvoid}, UInt64, Float64),
                         handle[], UInt64(seed), temperature))
        blocks = zeros(4, N_BLOCKS, length(systems))
        check(ctx, ccall((:pmgb_batch_results, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
                         handle[], blocks, C_NULL))
        R = PorousMaterials.UNIV_GAS_CONST
        kh = [mean(exp.(blocks[1, :, s] .- log(R * temperature * nb))) for s in 1:length(systems)]
        return_energies || return kh
        n = nb * N_BLOCKS
        u = zeros(2, n * length(systems))  # (U_vdw, U_es) per insertion, system after system
        check(ctx, ccall((:pmgb_batch_energies, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}), handle[], u))
        return kh, [u[:, (s - 1) * n + 1:s * n] for s in 1:length(systems)]
    finally
        ccall((:pmgb_batch_destroy, LIB), Cvoid, (Ptr{Cvoid},), handle[])
    end
end

end # module
