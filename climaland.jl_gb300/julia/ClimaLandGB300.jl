"""
    ClimaLandGB300

Julia binding of libclimaland_cuda (include/climaland_cuda.h): the soil column
step of a ClimaLand `RichardsModel` or `EnergyHydrology` on one GB300, behind
the existing model / `step!` interface.

The library takes the reference's column layout: for a scalar ClimaCore field
on a `Column` or extruded space, `parent(field)` holds the levels of a column
contiguously (level 1 = bottom), which is the layout `clm_set_state` expects
with `offsets[c] = (c - 1) * nlevels`.
"""
module ClimaLandGB300

const libclm = get(ENV, "CLIMALAND_CUDA_LIB", "libclimaland_cuda")

# ---- constants of include/climaland_cuda.h --------------------------------
const CLM_OK = Cint(0)
const CLM_MODEL_RICHARDS = Int32(0)
const CLM_MODEL_ENERGY_HYDROLOGY = Int32(1)
const CLM_PREC_FP64 = Int32(0)
const CLM_PREC_MIXED = Int32(1)
const CLM_NEWTON_FIXED = Int32(0)
const CLM_NEWTON_TOL = Int32(1)
const CLM_BC_FLUX = Int32(0)
const CLM_BC_FREE_DRAINAGE = Int32(1)
const CLM_BC_STATE = Int32(2)
const CLM_BC_FLUX_ADVECTIVE = Int32(3)
const CLM_BC_PRECIP_RUNOFF = Int32(4)
const CLM_BC_ATMOS = Int32(5)
const CLM_RUNOFF_NONE = Int32(0)
const CLM_RUNOFF_SURFACE = Int32(1)
const CLM_RUNOFF_TOPMODEL = Int32(2)
const CLM_CM_VAN_GENUCHTEN = Int32(0)
const CLM_CM_BROOKS_COREY = Int32(1)
const CLM_F_NFIELDS = 8
const CLM_RX_NFIELDS = 8
const CLM_AT_NFIELDS = 20
const CLM_AF_NFIELDS = 8

struct ClmEarthParams
    rho_l::Float64
    rho_i::Float64
    cp_l::Float64
    cp_i::Float64
    T_0::Float64
    T_freeze::Float64
    LH_f0::Float64
    grav::Float64
end

# Field order and types must match `clm_config` exactly.
mutable struct ClmConfig
    model::Int32
    ncol::Int32
    nlayers::Int32
    precision::Int32
    newton_mode::Int32
    max_iters::Int32
    newton_tol::Float64
    energy_norm_scale::Float64
    learned_guess::Int32
    bc_top_water::Int32
    bc_top_heat::Int32
    bc_bottom_water::Int32
    bc_bottom_heat::Int32
    kersten_alpha::Float64
    kersten_beta::Float64
    ice_impedance_omega::Float64
    visc_gamma::Float64
    visc_gamma_T_ref::Float64
    earth::ClmEarthParams
    phase_change::Int32
    pad0::Int32
    forcing_seed::UInt64
    cols_per_cta::Int32
    schedule::Int32
    graph::Int32
    hydrology_cm::Int32
    column_offset::Int64
    host_chunks::Int32
    runoff::Int32
    ClmConfig() = new()
end

function default_config()
    cfg = ClmConfig()
    ccall((:clm_config_default, libclm), Cvoid, (Ref{ClmConfig},), cfg)
    return cfg
end

"""
    earth_params(earth_param_set)

The `LandParameters` fields the step uses (src/shared_utilities/Parameters.jl).
"""
function earth_params(ps)
    LP = parentmodule(typeof(ps))
    return ClmEarthParams(
        LP.ρ_cloud_liq(ps), LP.ρ_cloud_ice(ps), LP.cp_l(ps), LP.cp_i(ps),
        LP.T_0(ps), LP.T_freeze(ps), LP.LH_f0(ps), LP.grav(ps),
    )
end

mutable struct Handle
    ptr::Ptr{Cvoid}
    ncol::Int
    ncells::Int
end

function check(h::Handle, rc)
    rc == CLM_OK && return nothing
    msg = unsafe_string(ccall((:clm_last_error, libclm), Cstring, (Ptr{Cvoid},), h.ptr))
    error("libclimaland_cuda error $rc: $msg")
end

function create(cfg::ClmConfig, ncells::Integer)
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:clm_create, libclm), Cint, (Ref{ClmConfig}, Ref{Ptr{Cvoid}}), cfg, out)
    rc == CLM_OK || error("clm_create failed with status $rc")
    h = Handle(out[], cfg.ncol, ncells)
    finalizer(h) do x
        x.ptr == C_NULL || ccall((:clm_destroy, libclm), Cvoid, (Ptr{Cvoid},), x.ptr)
        x.ptr = C_NULL
    end
    return h
end

set_geometry!(h::Handle, z_lo::Vector{Float64}, z_hi::Vector{Float64}, offsets::Union{Nothing, Vector{Int32}}) =
    check(h, ccall((:clm_set_geometry, libclm), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
        h.ptr, z_lo, z_hi, offsets === nothing ? C_NULL : offsets))

"""
    closure_rows(hcm)

Rows 5 and 6 of the parameter matrix and `cfg.hydrology_cm` for a
`vanGenuchten` (α, n) or `BrooksCorey` (ψb, c) closure
(src/standalone/Soil/retention_models.jl).
"""
function closure_rows(hcm)
    if hasproperty(hcm, :ψb)
        return hcm.ψb, hcm.c, CLM_CM_BROOKS_COREY
    end
    return hcm.α, hcm.n, CLM_CM_VAN_GENUCHTEN
end

"Per-column parameters as a (nparams × ncol) matrix, rows in `enum clm_param` order."
set_params!(h::Handle, p::Matrix{Float64}) =
    check(h, ccall((:clm_set_params, libclm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32),
        h.ptr, permutedims(p), size(p, 1)))

"""
    set_root_extraction!(h, r)

Root-extraction canopy values as a (CLM_RX_NFIELDS × ncol) matrix (rows:
canopy ψ, LAI, RAI, height, rooting depth, Weibull K_sat, ψ63, c), or
`nothing` to remove the source. From a ClimaLand `CanopyModel`: `p.canopy.hydraulics.ψ`,
`p.canopy.biomass.area_index.leaf` / `.root`, `canopy.biomass.height`,
`canopy.biomass.rooting_depth` and `canopy.hydraulics.parameters.conductivity_model`.
"""
set_root_extraction!(h::Handle, r::Union{Nothing, Matrix{Float64}}) =
    check(h, ccall((:clm_set_root_extraction, libclm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32),
        h.ptr, r === nothing ? C_NULL : permutedims(r), r === nothing ? 0 : size(r, 1)))

"Constants of the atmosphere-driven top boundary (`clm_atmos_params`)."
mutable struct ClmAtmosParams
    stefan::Float64
    gas_constant::Float64
    molmass_dryair::Float64
    molmass_water::Float64
    D_vapor::Float64
    LH_v0::Float64
    LH_s0::Float64
    cp_d::Float64
    cp_v::Float64
    T_triple::Float64
    press_triple::Float64
    von_karman::Float64
    Pr_0::Float64
    a_m::Float64
    a_h::Float64
    b_m::Float64
    b_h::Float64
    zeta_max::Float64
    iterations::Int32
    pad::Int32
end

function atmos_params_default()
    a = ClmAtmosParams(zeros(18)..., Int32(0), Int32(0))
    ccall((:clm_atmos_params_default, libclm), Cvoid, (Ref{ClmAtmosParams},), a)
    return a
end

"""
    set_atmos!(h, drivers; params = atmos_params_default())

Drivers of the atmosphere-driven top boundary (`cfg.bc_top_water =
cfg.bc_top_heat = CLM_BC_ATMOS`) as a (CLM_AT_NFIELDS × ncol) matrix, rows in
`enum clm_atmos_field` order: from a `PrescribedAtmosphere` /
`PrescribedRadiativeFluxes`, `p.drivers.P_liq, T, u, q, P, SW_d, LW_d`,
`atmos.h`, `atmos.gustiness`, then the soil's albedo parameters,
emissivity, z_0m, z_0b, d_ds, evap_p, evap_α. Call after each
`update_drivers!`; `nothing` removes them. The BC's runoff model is `cfg.runoff` (CLM_RUNOFF_*; TOPMODEL
also needs the f_max, f_over, R_sb parameter rows).
"""
function set_atmos!(h::Handle, d::Union{Nothing, Matrix{Float64}}; params = atmos_params_default())
    d === nothing && return check(h, ccall((:clm_set_atmos, libclm), Cint,
        (Ptr{Cvoid}, Ptr{ClmAtmosParams}, Ptr{Float64}, Int32), h.ptr, C_NULL, C_NULL, 0))
    check(h, ccall((:clm_set_atmos, libclm), Cint,
        (Ptr{Cvoid}, Ref{ClmAtmosParams}, Ptr{Float64}, Int32), h.ptr, params, permutedims(d), size(d, 1)))
end

"The boundary's diagnostics (lhf, shf, vapor_flux_liq, vapor_flux_ice, R_n, q_sfc, top water, top heat) as a (CLM_AF_NFIELDS × ncol) matrix."
function atmos_fluxes(h::Handle, ncol::Integer)
    out = Matrix{Float64}(undef, ncol, CLM_AF_NFIELDS)
    check(h, ccall((:clm_atmos_fluxes, libclm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Int32),
        h.ptr, out, CLM_AF_NFIELDS))
    return permutedims(out)
end

"Forcing descriptor for one boundary slot as a (CLM_F_NFIELDS × ncol) matrix."
set_bc!(h::Handle, slot::Integer, f::Matrix{Float64}) =
    check(h, ccall((:clm_set_bc, libclm), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32),
        h.ptr, slot, permutedims(f), size(f, 1)))

set_state!(h::Handle, ϑ_l, θ_i, ρe_int, ∫F_w, ∫F_e) =
    check(h, ccall((:clm_set_state, libclm), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h.ptr, ϑ_l, θ_i === nothing ? C_NULL : θ_i, ρe_int === nothing ? C_NULL : ρe_int,
        ∫F_w, ∫F_e === nothing ? C_NULL : ∫F_e))

get_state!(h::Handle, ϑ_l, θ_i, ρe_int, ∫F_w, ∫F_e) =
    check(h, ccall((:clm_get_state, libclm), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h.ptr, ϑ_l, θ_i === nothing ? C_NULL : θ_i, ρe_int === nothing ? C_NULL : ρe_int,
        ∫F_w, ∫F_e === nothing ? C_NULL : ∫F_e))

"""
    step!(h, t, dt, nsteps = 1)

`nsteps` IMEX ARS111 steps of the soil columns from time `t`: the body of
`step!(landsim)` (Simulations.jl:312-314) for a soil-only model.
"""
step!(h::Handle, t::Real, dt::Real, nsteps::Integer = 1) =
    check(h, ccall((:clm_step, libclm), Cint, (Ptr{Cvoid}, Float64, Float64, Int32),
        h.ptr, t, dt, nsteps))

"""
    step!(h, Y, t, dt)

Advance a ClimaLand state `Y` (FieldVector with `Y.soil.ϑ_l`, `Y.soil.θ_i`,
`Y.soil.ρe_int`, `Y.soil.∫F_vol_liq_water_dt`, `Y.soil.∫F_e_dt`) by one step
on the GPU, round-tripping through host memory.
"""
function step!(h::Handle, Y, t::Real, dt::Real)
    soil = Y.soil
    ϑ = vec(Array(parent(soil.ϑ_l)))
    eh = hasproperty(soil, :ρe_int)
    θi = eh ? vec(Array(parent(soil.θ_i))) : nothing
    ρe = eh ? vec(Array(parent(soil.ρe_int))) : nothing
    Fw = vec(Array(parent(soil.∫F_vol_liq_water_dt)))
    Fe = eh ? vec(Array(parent(soil.∫F_e_dt))) : nothing
    set_state!(h, ϑ, θi, ρe, Fw, Fe)
    step!(h, t, dt, 1)
    get_state!(h, ϑ, θi, ρe, Fw, Fe)
    copyto!(parent(soil.ϑ_l), ϑ)
    copyto!(parent(soil.∫F_vol_liq_water_dt), Fw)
    if eh
        copyto!(parent(soil.θ_i), θi)
        copyto!(parent(soil.ρe_int), ρe)
        copyto!(parent(soil.∫F_e_dt), Fe)
    end
    return Y
end

end # module
