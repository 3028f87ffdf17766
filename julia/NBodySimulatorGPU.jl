# NBodySimulatorGPU.jl - the Julia side of the drop-in: NBodySimulator.jl's
# own types and run_simulation, with the ODE right-hand side and the fused
# integration loops computed by libnbg.so (include/nbg.h) through ccall.
#
# This file is the binding a maintainer adds next to NBodySimulator.jl. It is
# not executed in this repository (no Julia runtime on the build or GPU
# machines); tests/test_julia_binding.py checks its structs against the C
# header field by field and every ccall against the declared prototypes.
#
# What it replaces (NBodySimulator.jl v1.15):
#   - the closures of SciMLBase.SecondOrderODEProblem(sim), src/nbody_to_ode.jl:460-536,
#     by one nbg_accel per right-hand-side evaluation (any SciML integrator);
#   - run_simulation(sim, VelocityVerlet(); dt), src/nbody_simulation_result.jl:468-487,
#     and its Langevin/EM branch (:489-492), by nbg_run (the whole loop on the GPU),
#     wrapped into the same SimulationResult through SciMLBase.build_solution;
#   - the histogram loops of rdf, :664-692, by nbg_rdf_histogram.
# Systems the library has no kernel for (a custom potential, BigFloat
# elements, CustomAccelerationSystem) return `nothing` from `descriptor`, and
# the entry points below leave them on the reference's CPU path.
module NBodySimulatorGPU

using NBodySimulator, SciMLBase, RecursiveArrayTools
using StochasticDiffEq: EM
using OrdinaryDiffEqSymplecticRK: VelocityVerlet
using NBodySimulator: NBodySimulation, PotentialNBodySystem, WaterSPCFw, ChargedParticles,
                      GravitationalSystem, CubicPeriodicBoundaryConditions,
                      PeriodicBoundaryConditions, InfiniteBox, NullThermostat, AndersenThermostat,
                      BerendsenThermostat, NoseHooverThermostat, LangevinThermostat,
                      LennardJonesParameters, ElectrostaticParameters, GravitationalParameters,
                      MagnetostaticParameters, SimulationResult

const libnbg = get(ENV, "NBG_LIBRARY", "libnbg.so")

const NBG_ABI_VERSION = Int32(1)
const NBG_SYSTEM_POTENTIAL, NBG_SYSTEM_WATER = Int32(0), Int32(1)
const NBG_POT_LJ, NBG_POT_EL, NBG_POT_GRAV, NBG_POT_MAG = UInt32(1), UInt32(2), UInt32(4), UInt32(8)
const NBG_BC_INFINITE, NBG_BC_CUBIC, NBG_BC_PERIODIC = Int32(0), Int32(1), Int32(2)
const NBG_THERMO_NULL, NBG_THERMO_ANDERSEN, NBG_THERMO_BERENDSEN, NBG_THERMO_NOSEHOOVER,
      NBG_THERMO_LANGEVIN = Int32(0), Int32(1), Int32(2), Int32(3), Int32(4)
const NBG_FLAG_LANGEVIN_BAOAB = Int32(4)
const NBG_ERR_UNSUPPORTED = Cint(-6)
const NBG_ERR_INDEX = Cint(-9)  # libnbg_debug.so (NBG_LIBRARY): a list or cell index out of range

# layout of nbg_system_desc (include/nbg.h), field for field
mutable struct NbgSystemDesc
    abi_version::Int32
    kind::Int32
    n::Int64
    mass::Ptr{Float64}
    charge::Ptr{Float64}
    dipole::Ptr{Float64}
    potentials::UInt32
    lj_epsilon::Float64
    lj_sigma::Float64
    lj_cutoff::Float64
    el_k::Float64
    el_cutoff::Float64
    el_eps_rf::Float64
    grav_G::Float64
    mag_mu_4pi::Float64
    water_rOH::Float64
    water_aHOH::Float64
    water_kb::Float64
    water_ka::Float64
    bc::Int32
    box::NTuple{6, Float64}
    thermostat::Int32
    thermo_T::Float64
    thermo_param::Float64
    kb::Float64
    seed::UInt64
    skin::Float64
    rebuild_every::Int32
    flags::Int32
end

NbgSystemDesc() = NbgSystemDesc(NBG_ABI_VERSION, NBG_SYSTEM_POTENTIAL, 0, C_NULL, C_NULL, C_NULL, UInt32(0),
                                0.0, 0.0, Inf, 0.0, Inf, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0,
                                NBG_BC_INFINITE, (0.0, 0.0, 0.0, 0.0, 0.0, 0.0),
                                NBG_THERMO_NULL, 0.0, 0.0, 1.38e-23, UInt64(0), 0.0, Int32(10), Int32(0))

# layout of nbg_run_stats
struct NbgRunStats
    steps::Int64
    list_builds::Int64
    kernel_launches::Int64
    device_ms::Float64
end

# layout of nbg_energies
struct NbgEnergies
    kinetic::Float64
    lennard_jones::Float64
    electrostatic::Float64
    bonds::Float64
    angles::Float64
    gravity::Float64
    potential::Float64
    total::Float64
    temperature::Float64
end

# layout of nbg_respa_stats
struct NbgRespaStats
    outer_mts::Int64
    outer_fallback::Int64
    judged::Int64
    judge_mean::Float64
    judge_max::Float64
    judge_last::Float64
end

# ---------------------------------------------------------------------------
# marshalling: what obtain_data_for_* (src/nbody_to_ode.jl:263-433) and
# get_masses (src/nbody_simulation_result.jl:121-139) extract, as plain values
# ---------------------------------------------------------------------------
is_plain(x::Real) = x isa Union{Float64, Float32, Integer}
is_plain(x::AbstractArray) = eltype(x) <: Union{Float64, Float32, Integer}
plain_body(b) = b isa NBodySimulator.WaterMolecule ? all(plain_body, (b.O, b.H1, b.H2)) :
                (is_plain(b.r) && is_plain(b.v) && is_plain(b.m))

# The descriptor and the arrays it points to (keep them alive across nbg_create),
# or `nothing` for a system the GPU library does not implement.
function descriptor(sim::NBodySimulation; skin = nothing, rebuild_every = 10, seed = 0, flags = 0)
    system = sim.system
    system isa Union{ChargedParticles, GravitationalSystem} && (system = PotentialNBodySystem(system))
    d = NbgSystemDesc()
    keep = Any[]
    masses = Vector{Float64}(NBodySimulator.get_masses(system))
    # BigFloat and other wide element types stay on the reference's CPU path
    all(is_plain, (sim.kb, sim.tspan...)) && all(plain_body, system.bodies) || return nothing
    push!(keep, masses)
    d.mass = pointer(masses)
    d.n = length(masses)
    if system isa WaterSPCFw
        all(is_plain, (system.mH, system.mO, system.qH, system.qO)) || return nothing
        d.kind = NBG_SYSTEM_WATER
        nm = length(system.bodies)
        q = Vector{Float64}(undef, 3nm)
        q[1:3:end] .= system.qO
        q[2:3:end] .= system.qH
        q[3:3:end] .= system.qH
        push!(keep, q)
        d.charge = pointer(q)
        lj, el, sp = system.lj_parameters, system.e_parameters, system.scpfw_parameters
        d.lj_epsilon, d.lj_sigma, d.lj_cutoff = lj.ϵ, lj.σ, lj.R
        d.el_k, d.el_cutoff, d.el_eps_rf = el.k, el.R, 1.0
        d.water_rOH, d.water_aHOH, d.water_kb, d.water_ka = sp.rOH, sp.aHOH, sp.kb, sp.ka
        d.potentials = NBG_POT_LJ | NBG_POT_EL
    elseif system isa PotentialNBodySystem
        d.kind = NBG_SYSTEM_POTENTIAL
        pots = system.potentials
        mask = UInt32(0)
        for (name, p) in pots
            name in (:lennard_jones, :electrostatic, :gravitational, :magnetostatic) || return nothing
            all(is_plain, (getfield(p, f) for f in fieldnames(typeof(p)))) || return nothing
        end
        if haskey(pots, :lennard_jones)
            p = pots[:lennard_jones]
            mask |= NBG_POT_LJ
            d.lj_epsilon, d.lj_sigma, d.lj_cutoff = p.ϵ, p.σ, p.R
        end
        if haskey(pots, :electrostatic)
            p = pots[:electrostatic]
            mask |= NBG_POT_EL
            d.el_k, d.el_cutoff, d.el_eps_rf = p.k, p.R, 1.0
            q = Float64[b.q for b in system.bodies]
            push!(keep, q)
            d.charge = pointer(q)
        end
        if haskey(pots, :gravitational)
            mask |= NBG_POT_GRAV
            d.grav_G = pots[:gravitational].G
        end
        if haskey(pots, :magnetostatic)
            mask |= NBG_POT_MAG
            d.mag_mu_4pi = pots[:magnetostatic].μ_4π
            mm = Vector{Float64}(undef, 3 * length(system.bodies))  # 3 x n, column-major
            for (i, b) in enumerate(system.bodies)
                mm[3i - 2:3i] .= b.mm
            end
            push!(keep, mm)
            d.dipole = pointer(mm)
        end
        d.potentials = mask
    else
        return nothing  # CustomAccelerationSystem: closures have no GPU kernel
    end
    bc = sim.boundary_conditions
    if bc isa CubicPeriodicBoundaryConditions
        d.bc, d.box = NBG_BC_CUBIC, (Float64(bc.L), 0.0, 0.0, 0.0, 0.0, 0.0)
    elseif bc isa PeriodicBoundaryConditions
        d.bc, d.box = NBG_BC_PERIODIC, Tuple(Float64.(bc.boundary))
    else
        d.bc = NBG_BC_INFINITE
    end
    th = sim.thermostat
    if th isa BerendsenThermostat
        d.thermostat, d.thermo_T, d.thermo_param = NBG_THERMO_BERENDSEN, th.T, th.τ
    elseif th isa NoseHooverThermostat
        d.thermostat, d.thermo_T, d.thermo_param = NBG_THERMO_NOSEHOOVER, th.T, th.τ
    elseif th isa AndersenThermostat
        d.thermostat, d.thermo_T, d.thermo_param = NBG_THERMO_ANDERSEN, th.T, th.ν
    elseif th isa LangevinThermostat
        d.thermostat, d.thermo_T, d.thermo_param = NBG_THERMO_LANGEVIN, th.T, th.γ
    else
        d.thermostat = NBG_THERMO_NULL
    end
    d.kb = sim.kb
    d.seed = UInt64(seed)
    cut = max((d.potentials & NBG_POT_LJ) != 0 ? d.lj_cutoff : 0.0,
              (d.potentials & NBG_POT_EL) != 0 ? d.el_cutoff : 0.0)
    d.skin = skin === nothing ? (isfinite(cut) ? 0.1 * cut : 0.0) : Float64(skin)
    d.rebuild_every = Int32(rebuild_every)
    d.flags = Int32(flags)
    return d, keep
end

# ---------------------------------------------------------------------------
# a context per simulation (nbg_create / nbg_destroy as the finalizer)
# ---------------------------------------------------------------------------
mutable struct Context
    ptr::Ptr{Cvoid}
    cols::Int   # state columns (n, or n + 1 with Nose-Hoover)
end

last_error(ctx::Context) = unsafe_string(@ccall libnbg.nbg_last_error(ctx.ptr::Ptr{Cvoid})::Cstring)
check(ctx::Context, st::Cint) = st == 0 || error("libnbg: ", last_error(ctx), " (status ", st, ")")

function Context(sim::NBodySimulation; device = 0, kwargs...)
    dk = descriptor(sim; kwargs...)
    dk === nothing && return nothing
    d, keep = dk
    out = Ref{Ptr{Cvoid}}(C_NULL)
    st = GC.@preserve keep d @ccall libnbg.nbg_create(d::Ref{NbgSystemDesc}, device::Cint,
                                                        out::Ref{Ptr{Cvoid}})::Cint
    st == NBG_ERR_UNSUPPORTED && return nothing
    st == 0 || error("nbg_create failed with status ", st)
    ctx = Context(out[], d.n + (d.thermostat == NBG_THERMO_NOSEHOOVER ? 1 : 0))
    finalizer(c -> (c.ptr != C_NULL && @ccall(libnbg.nbg_destroy(c.ptr::Ptr{Cvoid})::Cvoid); c.ptr = C_NULL), ctx)
    return ctx
end

# the Philox step counter of the Andersen / Langevin noise (checkpoints)
function get_step(ctx::Context)
    s = Ref{Int64}(0)
    check(ctx, @ccall libnbg.nbg_get_step(ctx.ptr::Ptr{Cvoid}, s::Ref{Int64})::Cint)
    return s[]
end
set_step!(ctx::Context, s::Integer) = check(ctx, @ccall libnbg.nbg_set_step(ctx.ptr::Ptr{Cvoid}, Int64(s)::Int64)::Cint)

# ---------------------------------------------------------------------------
# (a) the right-hand side drop-in: SecondOrderODEProblem(sim, Val(:gpu)) with
# f1!(dv, v, u, p, t) = one nbg_accel (3 x n Float64 matrices, no copy)
# ---------------------------------------------------------------------------
function SciMLBase.SecondOrderODEProblem(sim::NBodySimulation, ::Val{:gpu}; kwargs...)
    ctx = Context(sim; kwargs...)
    ctx === nothing && return SciMLBase.SecondOrderODEProblem(sim)  # stays on the reference's CPU path
    (u0, v0, n) = NBodySimulator.gather_bodies_initial_coordinates(sim)
    function f1!(dv, v, u, p, t)
        # the Nose-Hoover term writes the thermostat rate into v[:, n + 1],
        # as the reference's right-hand side does (thermostats.jl:126)
        st = @ccall libnbg.nbg_accel(ctx.ptr::Ptr{Cvoid}, dv::Ptr{Float64}, v::Ptr{Float64},
                                     u::Ptr{Float64}, t::Cdouble)::Cint
        check(ctx, st)
        return nothing
    end
    return SciMLBase.SecondOrderODEProblem(f1!, v0, u0, sim.tspan)
end

# ---------------------------------------------------------------------------
# (b) the fused loop: run_simulation(sim, GPUVelocityVerlet(); dt) and, with a
# LangevinThermostat, GPUEulerMaruyama() (the reference's EM on its SDE)
# ---------------------------------------------------------------------------
struct GPUVelocityVerlet end
struct GPUEulerMaruyama end

function NBodySimulator.run_simulation(sim::NBodySimulation, alg::Union{GPUVelocityVerlet, GPUEulerMaruyama};
                                       dt, save_everystep = true, save_every = nothing, device = 0, kwargs...)
    ctx = Context(sim; device = device, kwargs...)
    if ctx === nothing  # no GPU kernel for this system: the reference's own loop
        return sim.thermostat isa LangevinThermostat ? NBodySimulator.run_simulation(sim, EM(); dt = dt) :
               NBodySimulator.run_simulation(sim, VelocityVerlet(); dt = dt)
    end
    (u, v, n) = NBodySimulator.gather_bodies_initial_coordinates(sim)
    u = Matrix{Float64}(u)
    v = Matrix{Float64}(v)
    t0, t1 = sim.tspan
    steps = round(Int64, (t1 - t0) / dt)
    every = save_every === nothing ? (save_everystep ? 1 : 0) : Int(save_every)
    nsaved = every > 0 ? steps ÷ every + 1 + (steps % every == 0 ? 0 : 1) : 2
    nframes = (every > 0 ? steps ÷ every + 1 : 1) + 1  # room the call may use
    tu = Array{Float64}(undef, 3, ctx.cols, nframes)
    tv = similar(tu)
    stats = Ref{NbgRunStats}()
    st = @ccall libnbg.nbg_run(ctx.ptr::Ptr{Cvoid}, u::Ptr{Float64}, v::Ptr{Float64}, dt::Cdouble,
                               steps::Int64, every::Int64, tu::Ptr{Float64}, tv::Ptr{Float64},
                               stats::Ref{NbgRunStats})::Cint
    check(ctx, st)
    saved = every > 0 ? collect(0:every:steps) : [0]
    saved[end] == steps || push!(saved, steps)
    ts = [min(t0 + s * dt, t1) for s in saved]
    ts[end] = t1
    if sim.thermostat isa LangevinThermostat
        # the reference's SDE state hcat(u, v) (src/nbody_to_ode.jl:567-597)
        prob = SciMLBase.SDEProblem(sim)
        us = [hcat(tu[:, :, k], tv[:, :, k]) for k in 1:nsaved]
    else
        # SecondOrderODEProblem's state ArrayPartition(v, u) (src/nbody_to_ode.jl:490)
        prob = SciMLBase.SecondOrderODEProblem(sim)
        us = [ArrayPartition(tv[:, :, k], tu[:, :, k]) for k in 1:nsaved]
    end
    sol = SciMLBase.build_solution(prob, alg, ts, us; retcode = SciMLBase.ReturnCode.Success)
    return SimulationResult(sol, sim)
end

# energies of a state with the reference's definitions (nbody_simulation_result.jl:182-446)
function energies(ctx::Context, u::Matrix{Float64}, v::Matrix{Float64})
    e = Ref{NbgEnergies}()
    check(ctx, @ccall libnbg.nbg_energy(ctx.ptr::Ptr{Cvoid}, u::Ptr{Float64}, v::Ptr{Float64},
                                        e::Ref{NbgEnergies})::Cint)
    return e[]
end

# ---------------------------------------------------------------------------
# (c) rdf: the reference's histogram loops on the GPU, its normalisation unchanged
# ---------------------------------------------------------------------------
function rdf_gpu(sr::SimulationResult; maxbin = 1000)
    pbc = sr.simulation.boundary_conditions
    (_, indxs) = NBodySimulator.obtain_data_for_lennard_jones_interaction(sr.simulation.system)
    ts = sr.solution.t
    n = size(NBodySimulator.get_position(sr, ts[1]), 2)
    frames = Array{Float64}(undef, 3, n, length(ts))  # nframes x ncols x 3 in C order
    for (k, t) in enumerate(ts)
        frames[:, :, k] = NBodySimulator.get_position(sr, t)
    end
    idx = Int32.(indxs .- 1)
    hist = zeros(maxbin)
    st = @ccall libnbg.nbg_rdf_histogram(frames::Ptr{Float64}, length(ts)::Int64, n::Int64, idx::Ptr{Int32},
                                         length(idx)::Int64, Float64(pbc.L)::Cdouble, Int32(maxbin)::Int32,
                                         0::Cint, hist::Ptr{Float64})::Cint
    st == 0 || error("nbg_rdf_histogram failed with status ", st)
    dr = pbc.L / maxbin
    c = 4 / 3 * π * length(idx) / pbc.L^3
    rs = [(b - 1) * dr + dr / 2 for b in 1:maxbin]
    gr = [(hist[b] / (length(ts) * length(idx))) / (c * ((b * dr)^3 - ((b - 1) * dr)^3)) for b in 1:maxbin]
    return (rs, gr)
end

# ---------------------------------------------------------------------------
# the learned multiple-time-step add-on (WaterSPCFw on the list path)
# ---------------------------------------------------------------------------
function train_learned!(ctx::Context, u::Matrix{Float64}, v::Matrix{Float64}; temps = (280.0, 300.0, 320.0),
                        frames_per_T = 8, dt = 0.0005, steps = 4000)
    check(ctx, @ccall libnbg.nbg_ml_enable(ctx.ptr::Ptr{Cvoid})::Cint)
    check(ctx, @ccall libnbg.nbg_set_state(ctx.ptr::Ptr{Cvoid}, u::Ptr{Float64}, v::Ptr{Float64})::Cint)
    check(ctx, @ccall libnbg.nbg_ml_reserve(ctx.ptr::Ptr{Cvoid}, Int64(length(temps) * frames_per_T)::Int64)::Cint)
    rows = zeros(Int64, 2)
    for T in temps
        check(ctx, @ccall libnbg.nbg_set_thermostat_target(ctx.ptr::Ptr{Cvoid}, Int32(0)::Int32, T::Cdouble)::Cint)
        check(ctx, @ccall libnbg.nbg_advance(ctx.ptr::Ptr{Cvoid}, dt::Cdouble, Int64(1000)::Int64)::Cint)
        for f in 1:frames_per_T
            check(ctx, @ccall libnbg.nbg_advance(ctx.ptr::Ptr{Cvoid}, dt::Cdouble, Int64(100)::Int64)::Cint)
            check(ctx, @ccall libnbg.nbg_ml_collect(ctx.ptr::Ptr{Cvoid}, rows::Ptr{Int64})::Cint)
        end
    end
    check(ctx, @ccall libnbg.nbg_ml_normalize(ctx.ptr::Ptr{Cvoid})::Cint)
    check(ctx, @ccall libnbg.nbg_ml_init_params(ctx.ptr::Ptr{Cvoid}, UInt64(0)::UInt64, 0.1::Cdouble)::Cint)
    loss = zeros(2)
    check(ctx, @ccall libnbg.nbg_ml_train(ctx.ptr::Ptr{Cvoid}, Int64(steps)::Int64, Int32(2048)::Int32,
                                          1e-3::Cdouble, UInt64(1)::UInt64, loss::Ptr{Float64})::Cint)
    return loss
end

function respa!(ctx::Context; dt = 0.0005, inner = 4, outer = 1000, threshold = 0.02)
    stats = Ref{NbgRespaStats}()
    check(ctx, @ccall libnbg.nbg_respa_run(ctx.ptr::Ptr{Cvoid}, dt::Cdouble, Int32(inner)::Int32, Int64(outer)::Int64,
                                           threshold::Cdouble, Int32(0)::Int32, stats::Ref{NbgRespaStats})::Cint)
    return stats[]
end

export Context, GPUVelocityVerlet, GPUEulerMaruyama, rdf_gpu, get_step, set_step!, energies,
       train_learned!, respa!

end # module
