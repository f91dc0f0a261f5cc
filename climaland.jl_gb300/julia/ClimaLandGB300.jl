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
const CLM_GUESS_NONE = Int32(0)
const CLM_GUESS_NETWORK = Int32(1)
const CLM_GUESS_EXTRAPOLATE = Int32(2)
const CLM_TOL_TILES = Int32(0)
const CLM_TOL_REGROUP = Int32(1)
const CLM_TOL_SPLIT = Int32(2)
const CLM_TOL_AUTO = Int32(3)
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
    tol_regroup::Int32
    pad1::Int32
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
    universal_functions::Int32   # CLM_UF_BUSINGER or CLM_UF_GRYANIK
    gryanik_b_m::Float64
    gryanik_b_h::Float64
end

const CLM_UF_BUSINGER = Int32(0)
const CLM_UF_GRYANIK = Int32(1)

function atmos_params_default()
    a = ClmAtmosParams(zeros(18)..., Int32(0), Int32(0), 0.0, 0.0)
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

"""
    set_faces!(h, z_faces)

Per-layer geometry of stretched columns (`Column(; dz_tuple)`,
`global_domain`): each column's n + 1 face coordinates, bottom to top, in the
layout of a face field (`parent(coordinate_field(face_space(space)).z)`),
or `nothing` for uniform layers.
"""
set_faces!(h::Handle, z_faces::Union{Nothing, Vector{Float64}}) =
    check(h, ccall((:clm_set_faces, libclm), Cint, (Ptr{Cvoid}, Ptr{Float64}),
        h.ptr, z_faces === nothing ? C_NULL : z_faces))

"The handle's work on a caller's CUDA stream (e.g. `CUDA.stream().handle`), or `nothing` for its own."
set_stream!(h::Handle, stream) =
    check(h, ccall((:clm_set_stream, libclm), Cint, (Ptr{Cvoid}, Ptr{Cvoid}),
        h.ptr, stream === nothing ? C_NULL : stream))

"""
    set_state_device!(h, ϑ_l, θ_i, ρe_int, ∫F_w, ∫F_e)

The state from device memory: `pointer(parent(field))` of CuArray-backed
fields (reference layout); copied on the handle's stream.
"""
set_state_device!(h::Handle, ϑ_l, θ_i, ρe_int, ∫F_w, ∫F_e) =
    check(h, ccall((:clm_set_state_device, libclm), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
        h.ptr, ϑ_l, θ_i === nothing ? C_NULL : θ_i, ρe_int === nothing ? C_NULL : ρe_int,
        ∫F_w, ∫F_e === nothing ? C_NULL : ∫F_e))

get_state_device!(h::Handle, ϑ_l, θ_i, ρe_int, ∫F_w, ∫F_e) =
    check(h, ccall((:clm_get_state_device, libclm), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
        h.ptr, ϑ_l, θ_i === nothing ? C_NULL : θ_i, ρe_int === nothing ? C_NULL : ρe_int,
        ∫F_w, ∫F_e === nothing ? C_NULL : ∫F_e))

"Column budgets `total_water`, `total_energy` of the current state (rre.jl:502-511, energy_hydrology.jl:1282-1320)."
function budgets(h::Handle)
    W = Vector{Float64}(undef, h.ncol)
    E = Vector{Float64}(undef, h.ncol)
    check(h, ccall((:clm_get_budgets, libclm), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
        h.ptr, W, E))
    return W, E
end

"Per-column status flags (CLM_COL_*) and Newton iterations of the last step call."
function status(h::Handle)
    flags = Vector{UInt32}(undef, h.ncol)
    iters = Vector{Int32}(undef, h.ncol)
    check(h, ccall((:clm_get_status, libclm), Cint, (Ptr{Cvoid}, Ptr{UInt32}, Ptr{Int32}),
        h.ptr, flags, iters))
    return flags, iters
end

# ---- closure level: the functions ClimaLand hands to ClimaTimeSteppers ----
# Each takes the handle's current state (set_state! / set_state_device!) at
# time t and writes host arrays in the reference layout.

"""
    update_aux!(h, t; K, ψ, θ_l, T, κ, Tf, bc)

`make_update_aux` + boundary fluxes (rre.jl:368-380, 111-149;
energy_hydrology.jl:722-814, 273-298): per-cell aux fields (any may be
`nothing`) and the boundary fluxes `bc` (4 × ncol: top water, top heat,
bottom water, bottom heat).
"""
function update_aux!(h::Handle, t::Real; K = nothing, ψ = nothing, θ_l = nothing, T = nothing,
                     κ = nothing, Tf = nothing, bc = nothing)
    p(x) = x === nothing ? C_NULL : x
    check(h, ccall((:clm_update_aux, libclm), Cint,
        (Ptr{Cvoid}, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}, Ptr{Float64}),
        h.ptr, t, p(K), p(ψ), p(θ_l), p(T), p(κ), p(Tf), p(bc)))
end

"`make_exp_tendency` (models.jl:279-287) into host arrays dY (per cell) and d∫F (per column)."
exp_tendency!(h::Handle, t::Real, dϑ, dθ_i, dρe, d∫F_w, d∫F_e) =
    check(h, ccall((:clm_exp_tendency, libclm), Cint,
        (Ptr{Cvoid}, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h.ptr, t, dϑ, dθ_i === nothing ? C_NULL : dθ_i, dρe === nothing ? C_NULL : dρe,
        d∫F_w, d∫F_e === nothing ? C_NULL : d∫F_e))

"`make_compute_imp_tendency` (implicit_timestepping.jl:25-28; rre.jl:161-203, energy_hydrology.jl:363-425) after the cache update."
imp_tendency!(h::Handle, t::Real, dϑ, dθ_i, dρe, d∫F_w, d∫F_e) =
    check(h, ccall((:clm_imp_tendency, libclm), Cint,
        (Ptr{Cvoid}, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h.ptr, t, dϑ, dθ_i === nothing ? C_NULL : dθ_i, dρe === nothing ? C_NULL : dρe,
        d∫F_w, d∫F_e === nothing ? C_NULL : d∫F_e))

"""
    jacobian!(h, t, dtγ, W_vv, W_ev, W_ee)

`make_compute_jacobian` (rre.jl:391-458; energy_hydrology.jl:466-576):
W = dtγ ∂T/∂Y - I as tridiagonal blocks, 3 values per cell (lower, diagonal,
upper): the rows of the `BidiagonalMatrixRow`/`TridiagonalMatrixRow`
entries of ClimaCore's FieldMatrix at (@name(soil.ϑ_l), @name(soil.ϑ_l)),
(@name(soil.ρe_int), @name(soil.ϑ_l)) and (@name(soil.ρe_int), @name(soil.ρe_int)).
"""
jacobian!(h::Handle, t::Real, dtγ::Real, W_vv, W_ev, W_ee) =
    check(h, ccall((:clm_jacobian, libclm), Cint,
        (Ptr{Cvoid}, Float64, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        h.ptr, t, dtγ, W_vv, W_ev === nothing ? C_NULL : W_ev, W_ee === nothing ? C_NULL : W_ee))

"The block solve of initialize_jacobian's FieldMatrixSolver (implicit_timestepping.jl:160-171): W δ = f per column."
solve!(h::Handle, W_vv, W_ev, W_ee, f_v, f_e, δ_v, δ_e) =
    check(h, ccall((:clm_solve, libclm), Cint,
        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
         Ptr{Float64}),
        h.ptr, W_vv, W_ev === nothing ? C_NULL : W_ev, W_ee === nothing ? C_NULL : W_ee, f_v,
        f_e === nothing ? C_NULL : f_e, δ_v, δ_e === nothing ? C_NULL : δ_e))

"""
    closures(h)

The model closures `Simulations.jl:171-199` assembles into
`CTS.ClimaODEFunction(; T_exp!, T_imp! = ODEFunction(T_imp!; jac_prototype, Wfact), cache_imp!)`,
evaluated by the library on the soil state. Each takes ClimaLand's
arguments and moves `Y.soil` through host memory:
  T_imp!(dY, Y, p, t)          make_compute_imp_tendency
  T_exp!(dY, Y, p, t)          make_exp_tendency
  cache_imp!(Y, p, t)          make_update_implicit_cache (aux into p.soil)
  Wfact!(W, Y, p, dtγ, t)      make_compute_jacobian (W: a NamedTuple of
                               three 3 × ncells matrices vv, ev, ee)
"""
function closures(h::Handle)
    eh(Y) = hasproperty(Y.soil, :ρe_int)
    host(f) = vec(Array(parent(f)))
    function load!(Y)
        s = Y.soil
        set_state!(h, host(s.ϑ_l), eh(Y) ? host(s.θ_i) : nothing, eh(Y) ? host(s.ρe_int) : nothing,
                   host(s.∫F_vol_liq_water_dt), eh(Y) ? host(s.∫F_e_dt) : nothing)
    end
    function store!(dY, dv, dti, de, dfw, dfe)
        s = dY.soil
        copyto!(parent(s.ϑ_l), dv)
        copyto!(parent(s.∫F_vol_liq_water_dt), dfw)
        if dti !== nothing
            copyto!(parent(s.θ_i), dti)
            copyto!(parent(s.ρe_int), de)
            copyto!(parent(s.∫F_e_dt), dfe)
        end
        return nothing
    end
    function tendency(f)
        return function (dY, Y, p, t)
            load!(Y)
            nc, e = h.ncells, eh(Y)
            dv, dfw = zeros(nc), zeros(h.ncol)
            dti, de, dfe = e ? zeros(nc) : nothing, e ? zeros(nc) : nothing, e ? zeros(h.ncol) : nothing
            f(h, t, dv, dti, de, dfw, dfe)
            store!(dY, dv, dti, de, dfw, dfe)
        end
    end
    function cache_imp!(Y, p, t)
        load!(Y)
        nc = h.ncells
        K, ψ = zeros(nc), zeros(nc)
        T = eh(Y) ? zeros(nc) : nothing
        update_aux!(h, t; K, ψ, T)
        copyto!(parent(p.soil.ψ), ψ)
        eh(Y) && copyto!(parent(p.soil.T), T)
        return nothing
    end
    function Wfact!(W, Y, p, dtγ, t)
        load!(Y)
        jacobian!(h, t, dtγ, W.vv, eh(Y) ? W.ev : nothing, eh(Y) ? W.ee : nothing)
        return nothing
    end
    return (; T_imp! = tendency(imp_tendency!), T_exp! = tendency(exp_tendency!), cache_imp!, Wfact!)
end

"""
    GB300Simulation(landsim, h)

A `LandSimulation` whose soil step runs on the GPU: `step!(sim)` advances
`landsim._integrator`'s state `u` by one step of size `dt` from `t` through
the handle (the body of `step!(landsim)`, Simulations.jl:312-314, for a
soil-only model), then advances the integrator's time, so that the
simulation's callbacks and diagnostics see the same `u` and `t`.
"""
struct GB300Simulation{S}
    landsim::S
    h::Handle
end

function step!(sim::GB300Simulation)
    integ = sim.landsim._integrator
    step!(sim.h, integ.u, integ.t, integ.dt)
    integ.t += integ.dt
    return sim
end

end # module
