"""
    PorousMaterialsGB300

`ccall` binding of libpmgb (the sm_103a Widom-insertion / energy-grid library, C ABI in
include/pmgb.h) for PorousMaterials.jl v0.4.  It provides drop-in bodies for

  * `henry_coefficient(crystal, molecule, temperature, ljff; insertions_per_volume,
     verbose, ewald_precision, autosave, filename_comment)`      (src/henry.jl:34-181)
  * `energy_grid(crystal, molecule, ljff; resolution, units, center, verbose)` for
     single-site probes                                          (src/grid.jl:291-362)

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
Drop-in for `henry_coefficient` (src/henry.jl:34-181): the same set-up, statistics, result
keys, units and autosave; the insertions run on the GPU.  `seed` makes a run reproducible;
`refine_tail` (default 1e-3) re-evaluates in high precision the insertions that carry all but that
fraction of each block's Boltzmann weight, which keeps K_H within 1e-6 of an FP64 evaluation.
"""
function henry_coefficient(crystal::Crystal, molecule::Molecule, temperature::Float64,
                           ljforcefield::LJForceField; insertions_per_volume::Union{Int, Float64}=200,
                           verbose::Bool=true, ewald_precision::Float64=1e-6, autosave::Bool=true,
                           filename_comment::AbstractString="", seed::UInt64=rand(UInt64),
                           ctx::Context=default_context(), refine_tail::Float64=1e-3, return_energies::Bool=false)
    assert_P1_symmetry(crystal)
    time_start = time()
    nb_insertions = max(N_BLOCKS, ceil(Int, insertions_per_volume * crystal.box.Ω))
    nb_insertions_per_block = ceil(Int, nb_insertions / N_BLOCKS)
    repfactors = replication_factors(crystal.box, ljforcefield)
    crystal = replicate(crystal, repfactors)
    molecule = Frac(molecule, crystal.box)
    charged_system = has_charges(crystal) && has_charges(molecule)
    ρ = crystal_density(crystal)
    eparams = charged_system ? setup_Ewald_sum(crystal.box, sqrt(ljforcefield.r²_cutoff);
                                               ϵ=ewald_precision, verbose=verbose) : nothing
    sys = GPUSystem(ctx, crystal, molecule, ljforcefield; eparams=eparams, refine_tail=refine_tail)
    blocks = widom_blocks(sys, nb_insertions_per_block, temperature; seed=seed)

    henry_coefficients = exp.(blocks[1, :] .- log(PorousMaterials.UNIV_GAS_CONST * temperature *
                                                    nb_insertions_per_block))
    avg_vdw = blocks[2, :]
    avg_es = charged_system ? blocks[3, :] : zeros(N_BLOCKS)
    err_kh = 2.0 * std(henry_coefficients) / sqrt(N_BLOCKS)
    err_vdw = 2.0 * std(avg_vdw) / sqrt(N_BLOCKS)
    err_es = 2.0 * std(avg_es) / sqrt(N_BLOCKS)
    K_TO_KJ = PorousMaterials.K_TO_KJ_PER_MOL

    results = Dict{String, Any}()
    results["henry coefficient [mol/(m³-bar)]"] = mean(henry_coefficients)
    results["xtal"] = crystal.name
    results["henry coefficient [mmol/(g-bar)]"] = results["henry coefficient [mol/(m³-bar)]"] / ρ
    results["err henry coefficient [mmol/(g-bar)]"] = err_kh / ρ
    results["henry coefficient [mol/(kg-Pa)]"] = results["henry coefficient [mmol/(g-bar)]"] / 100000.0
    results["⟨U, vdw⟩ (K)"] = mean(avg_vdw)
    results["⟨U, es⟩ (K)"] = mean(avg_es)
    results["⟨U⟩ (K)"] = results["⟨U, vdw⟩ (K)"] + results["⟨U, es⟩ (K)"]
    results["⟨U⟩ (kJ/mol)"] = results["⟨U⟩ (K)"] * K_TO_KJ
    results["⟨U, vdw⟩ (kJ/mol)"] = results["⟨U, vdw⟩ (K)"] * K_TO_KJ
    results["err ⟨U, vdw⟩ (kJ/mol)"] = err_vdw * K_TO_KJ
    results["⟨U, es⟩ (kJ/mol)"] = results["⟨U, es⟩ (K)"] * K_TO_KJ
    results["err ⟨U, es⟩ (kJ/mol)"] = err_es * K_TO_KJ
    results["Qst (kJ/mol)"] = -results["⟨U⟩ (kJ/mol)"] + temperature * K_TO_KJ
    results["err Qst (kJ/mol)"] = (err_vdw + err_es) * K_TO_KJ
    results["elapsed time (min)"] = (time() - time_start) / 60
    if autosave
        isdir(rc[:paths][:simulations]) || mkdir(rc[:paths][:simulations])
        savename = joinpath(rc[:paths][:simulations],
                            henry_result_savename(crystal, molecule, temperature, ljforcefield,
                                                  insertions_per_volume, comment=filename_comment))
        @save savename results
        verbose && println("\tResults saved in: ", savename)
    end
    if verbose
        for key in ["henry coefficient [mmol/(g-bar)]", "⟨U, vdw⟩ (kJ/mol)", "⟨U, es⟩ (kJ/mol)", "Qst (kJ/mol)"]
            @printf("\t%s = %f +/- %f\n", key, results[key], results["err " * key])
        end
    end
    return results
end

"""
Drop-in for `energy_grid` (src/grid.jl:291-362) with a single-site probe (no rotations).
"""
function energy_grid(crystal::Crystal, molecule::Molecule{Cart}, ljforcefield::LJForceField;
                     resolution::Union{Float64, Tuple{Int, Int, Int}}=1.0, units::Symbol=:kJ_mol,
                     center::Bool=false, verbose::Bool=true, ctx::Context=default_context())
    assert_P1_symmetry(crystal)
    units in (:kJ_mol, :K) || error("Pass :kJ_mol or :K for units of kJ/mol or K, respectively.")
    needs_rotations(molecule) && error("the GPU energy grid takes single-site probes")
    n_pts = isa(resolution, Tuple{Int, Int, Int}) ? resolution : required_n_pts(crystal.box, resolution)
    repfactors = replication_factors(crystal.box, ljforcefield)
    sc = replicate(crystal, repfactors)
    sys = GPUSystem(ctx, sc, Frac(molecule, sc.box), ljforcefield)
    factor = units == :kJ_mol ? PorousMaterials.K_TO_KJ_PER_MOL : 1.0
    data = Array{Float32}(undef, n_pts...)     # column-major: i fastest, as the ABI writes
    check(ctx, ccall((:pmgb_energy_grid, LIB), Cint,
        (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Float64, Ptr{Float32}),
        sys.ptr, Int32[n_pts...], Int32[repfactors...], factor, data))
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
                      ctx::Context=default_context(), refine_tail::Float64=1e-3)
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
