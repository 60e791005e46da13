"""
    EnsembleGB300

SciML ensemble algorithm that runs every trajectory of an `EnsembleProblem` on
one GB300 through `libode_b200.so` (C ABI in `include/ode_gb300.h`).

    using OrdinaryDiffEq, EnsembleGB300
    prob = ODEProblem(GB300Model(:robertson), [1.0, 0.0, 0.0], (0.0, 1e5), [0.04, 3e7, 1e4])
    eprob = EnsembleProblem(prob; prob_func = (prob, ctx) -> remake(prob; p = prob.p .* 2.0 .^ (2rand(ctx.rng, 3) .- 1)))
    sim = solve(eprob, Rodas5P(), EnsembleGB300(); trajectories = 100_000,
                saveat = 10 .^ range(-5, 5; length = 20), reltol = 1e-6, abstol = 1e-10)

Right-hand sides are device functions: compiled into the library and named by
`GB300Model` (:linear, :lorenz, :robertson, :duffing_chain, :brusselator_1d,
...), or registered at run time as CUDA C++ source with `register_model`
(the library compiles them with NVRTC); arbitrary Julia closures cannot run
on the device.

    lv = register_model("""
        template <class T, class P> __device__ void lv_f(T* du, const T* u, const P* p, double t) {
            du[0] = p[0] * u[0] - p[1] * u[0] * u[1];
            du[1] = p[3] * u[0] * u[1] - p[2] * u[1];
        }""", :lv, 2, 4)
    prob = ODEProblem(lv, [1.0, 1.0], (0.0, 10.0), [1.5, 1.0, 3.0, 1.0])
"""
module EnsembleGB300Ext

using SciMLBase
import OrdinaryDiffEqTsit5: Tsit5
import OrdinaryDiffEqVerner: Vern7
import OrdinaryDiffEqRosenbrock: Rodas5P, Rosenbrock23
import OrdinaryDiffEqCore: CompositeAlgorithm, AutoSwitch, PIController

export EnsembleGB300, GB300Model, GB300Callback, register_model

const LIB = get(ENV, "ODE_GB300_LIB", joinpath(@__DIR__, "..", "lib", "libode_b200.so"))

const MODEL_IDS = Dict(:linear => 0, :lorenz => 1, :robertson => 2, :duffing_chain => 3, :brusselator_1d => 4,
                       :bouncing_ball => 5, :van_der_pol => 6, :pk_one_compartment => 7, :forced_duffing => 8)
const N_PARAMS = Dict(0 => 1, 1 => 3, 2 => 3, 3 => 3, 4 => 3, 5 => 3, 6 => 1, 7 => 3, 8 => 5)

"""
    GB300Callback(; interp_points = 10, max_events = 16)

Turns on the model's registered callback (its condition and affect are device
code compiled with the model): the ContinuousCallback of `:bouncing_ball`, or
the DiscreteCallback of `:pk_one_compartment` (condition `t in tstops`, the
dose times passed as `solve`'s `tstops`); pass it as `callback` to `solve`.
Each firing adds two saves (before and after its affect).
"""
struct GB300Callback
    interp_points::Int
    max_events::Int
end
GB300Callback(; interp_points = 10, max_events = 16) = GB300Callback(interp_points, max_events)

"""Marker right-hand side naming a model compiled into the library or registered with `register_model`."""
struct GB300Model
    name::Symbol
end
(m::GB300Model)(du, u, p, t) = error("GB300Model($(m.name)) only runs on the device")

"""
    register_model(source, name, n_states, n_params; jac = false, tgrad = false, nonautonomous = false)

Registers a right-hand side written as CUDA C++ (`ode_register_model`): the
source defines `template <class T, class P> __device__ void NAME_f(T* du, const
T* u, const P* p, double t)` and, with `jac`/`tgrad`, `NAME_jac(T* J, ...)`
(row-major) and `NAME_tgrad(T* dT, ...)`; without `jac` the Rosenbrock methods
differentiate `NAME_f` by forward-mode AD on the device.  Returns a
`GB300Model` usable as the `f` of an `ODEProblem`.
"""
function register_model(source::AbstractString, name::Symbol, n_states::Integer, n_params::Integer;
                        jac::Bool = false, tgrad::Bool = false, nonautonomous::Bool = false)
    flags = Int32((jac ? 1 : 0) | (tgrad ? 2 : 0) | (nonautonomous ? 4 : 0))
    id = Ref{Int32}(0)
    st = ccall((:ode_register_model, LIB), Cint, (Cstring, Cstring, Int32, Int32, Int32, Ref{Int32}),
               source, String(name), Int32(n_states), Int32(n_params), flags, id)
    st == 0 || error("ode_register_model: " * unsafe_string(ccall((:ode_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL)))
    MODEL_IDS[name] = Int(id[])
    N_PARAMS[Int(id[])] = Int(n_params)
    return GB300Model(name)
end

struct EnsembleGB300 <: SciMLBase.EnsembleAlgorithm
    precision::Symbol      # :fp64 or :mixed
    device::Int
    lanes_per_traj::Int
    scheduler::Int
end
EnsembleGB300(; precision = :fp64, device = 0, lanes_per_traj = 0, scheduler = 0) =
    EnsembleGB300(precision, device, lanes_per_traj, scheduler)

# Mirrors of the C structs (include/ode_gb300.h).
struct ProblemDesc
    model_id::Int32; alg_id::Int32; n_states::Int32; n_params::Int32; precision::Int32; reserved::Int32
end
mutable struct Options
    reltol::Float64; abstol::Float64; dtmax::Float64; dtmin::Float64; dt::Float64; maxiters::Int64
    save_start::Int32; save_end::Int32; save_end_user::Int32; saveat_scalar::Int32; nsave::Int32
    saveat_per_traj::Int32; qmax_first_step::Float64; qmax::Float64; lanes_per_traj::Int32
    scheduler::Int32; block_size::Int32; ir_sweeps::Int32; save_everystep::Int32; max_step_saves::Int32
    callback::Int32; interp_points::Int32; max_events::Int32; ntstops::Int32; tstops::Ptr{Float64}
    max_jac_age::Int32; isoutofdomain::Int32; jac_reuse_gamma_tol::Float64
    nsave_idxs::Int32; reserved3::Int32; save_idxs::Ptr{Int32}
    adaptive::Int32; forward_only::Int32
    controller_given::Int32; force_dtmin::Int32
    beta1::Float64; beta2::Float64; qoldinit::Float64; qmin::Float64; gamma::Float64
    qsteady_min::Float64; qsteady_max::Float64
    abstol_vec::Ptr{Float64}; reltol_vec::Ptr{Float64}
end
# the knobs of solve(...; controller = PIController(beta1, beta2; qoldinit, qmin, qmax,
# qmax_first_step, gamma, qsteady_min, qsteady_max)): beta1, beta2 and qoldinit on the
# controller, the rest as overrides in its `basic` (a NamedTuple until resolved)
_knob(b::NamedTuple, k) = haskey(b, k) && b[k] !== nothing ? Float64(b[k]) : NaN
_knob(b, k) = Float64(getfield(b, k))
function controller_knobs(c)
    c === nothing && return (Int32(0), fill(NaN, 7), 0.0, 0.0)
    c isa PIController || error("EnsembleGB300 runs the PI controller: pass controller = PIController(...)")
    b = c.basic
    qm, qmf = _knob(b, :qmax), _knob(b, :qmax_first_step)
    return (Int32(1), [Float64(c.beta1), Float64(c.beta2), Float64(c.qoldinit), _knob(b, :qmin), _knob(b, :gamma),
                       _knob(b, :qsteady_min), _knob(b, :qsteady_max)],
            isnan(qm) ? 0.0 : qm, isnan(qmf) ? 0.0 : qmf)
end
# the W-method Jacobian reuse knobs of Rosenbrock23(max_jac_age, jac_reuse_gamma_tol)
jac_reuse(alg::Rosenbrock23) = (Int32(alg.max_jac_age), Float64(alg.jac_reuse_gamma_tol))
jac_reuse(alg) = (Int32(1), 0.03)
struct Stats
    nf::Int64; njacs::Int64; nw::Int64; nsolve::Int64; naccept::Int64; nreject::Int64
end

alg_id(::Tsit5) = Int32(0)
alg_id(::Vern7) = Int32(1)
alg_id(::Rodas5P) = Int32(2)
alg_id(::Rosenbrock23) = Int32(3)
# AutoTsit5(Rosenbrock23()) with the default AutoSwitch (the composite compiled in)
function alg_id(alg::CompositeAlgorithm)
    cf = alg.choice_function
    ok = length(alg.algs) == 2 && alg.algs[1] isa Tsit5 && alg.algs[2] isa Rosenbrock23 && cf isa AutoSwitch &&
         cf.maxstiffstep == 10 && cf.maxnonstiffstep == 3 && cf.nonstifftol == 9 // 10 && cf.stifftol == 9 // 10 &&
         cf.dtfac == 2 && !cf.stiffalgfirst && cf.switch_max == 5
    ok || error("EnsembleGB300 runs AutoTsit5(Rosenbrock23()) with the default AutoSwitch only")
    return Int32(4)
end

const RETCODES = (SciMLBase.ReturnCode.Default, SciMLBase.ReturnCode.Success, SciMLBase.ReturnCode.MaxIters,
                  SciMLBase.ReturnCode.DtNaN, SciMLBase.ReturnCode.DtLessThanMin, SciMLBase.ReturnCode.Unstable,
                  SciMLBase.ReturnCode.Terminated, SciMLBase.ReturnCode.Terminated,
                  SciMLBase.ReturnCode.InitialFailure)

"""
Interpolation of a dense GB300 solve (the reference's dense = true): sol(t)
evaluates the method's interpolant on the saved steps on the device
(ode_dense_eval_deriv; sol(t, Val{1}) and, for Tsit5 and Rodas5P, sol(t, Val{2}) too), as ode_interpolation does on the host.  Holds one
trajectory's saves t (ns), u (n x ns) and interpolation vectors k (n x nk x ns).
"""
struct GB300DenseInterpolation <: SciMLBase.AbstractDiffEqInterpolation
    model::Int32
    alg::Int32
    p::Vector{Float64}
    device::Int
    t::Vector{Float64}
    u::Matrix{Float64}
    k::Array{Float64, 3}
end

function (id::GB300DenseInterpolation)(tvals, idxs, deriv, p, continuity::Symbol = :left)
    order = deriv == Val{0} ? 0 : deriv == Val{1} ? 1 : deriv == Val{2} ? 2 : deriv == Val{3} ? 3 :
            error("GB300 dense output evaluates the solution (Val{0}) and its derivatives Val{1} to Val{3}")
    tq = tvals isa Number ? [Float64(tvals)] : collect(Float64, tvals)
    n, ns, nq = size(id.u, 1), length(id.t), length(tq)
    d = ProblemDesc(id.model, id.alg, n, length(id.p), 0, 0)
    out = zeros(n, nq)   # [(r*n + i)*N + j] with N = 1 -> out[i, r]
    continuity in (:left, :right) || error("continuity: :left or :right")
    status = ccall((:ode_dense_eval_ex, LIB), Cint,
                   (Ptr{Cvoid}, Ref{ProblemDesc}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Int32}, Int32, Int32, Ptr{Float64}, Int32, Int32, Int32, Ptr{Float64}),
                   handle(id.device), d, 1, id.p, id.t, id.u, id.k, Int32[ns], ns, nq, tq, 0, order,
                   Int32(continuity === :right), out)
    status == 0 || error("ode_dense_eval_ex: ", unsafe_string(ccall((:ode_last_error, LIB), Cstring, (Ptr{Cvoid},), handle(id.device))))
    vals = [idxs === nothing ? out[:, r] : out[idxs, r] for r in 1:nq]
    tvals isa Number ? vals[1] : vals
end

const HANDLES = Dict{Int, Ptr{Cvoid}}()
function handle(dev)
    get!(HANDLES, dev) do
        # the struct mirrors above must match the library's layout
        ccall((:ode_options_size, LIB), Csize_t, ()) == sizeof(Options) &&
            ccall((:ode_problem_desc_size, LIB), Csize_t, ()) == sizeof(ProblemDesc) ||
            error("EnsembleGB300: Options/ProblemDesc do not match the library's ode_options/ode_problem_desc")
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:ode_create, LIB), Cint, (Cint, Csize_t, Ref{Ptr{Cvoid}}), dev, 0, h)
        rc == 0 || error("ode_create failed: ", unsafe_string(ccall((:ode_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL)))
        h[]
    end
end

function SciMLBase.__solve(eprob::SciMLBase.AbstractEnsembleProblem,
                           alg::Union{Tsit5, Vern7, Rodas5P, Rosenbrock23, CompositeAlgorithm},
                           ens::EnsembleGB300; trajectories, saveat = Float64[], reltol = 1e-3, abstol = 1e-6,
                           dt = 0.0, dtmax = 0.0, dtmin = 0.0, maxiters = 1_000_000, save_start = nothing,
                           save_end = nothing, save_everystep = isempty(saveat), max_step_saves = 1024, seed = 0,
                           save_idxs = nothing, adaptive = true, controller = nothing, force_dtmin = false,
                           isoutofdomain = nothing, callback = nothing,
                           dense = save_everystep && isempty(saveat) && save_idxs === nothing,
                           tstops = Float64[], kwargs...)
    t0 = time()
    N = trajectories
    probs = [eprob.prob_func(eprob.prob, SciMLBase.EnsembleContext(i, 1, seed)) for i in 1:N]
    f = probs[1].f.f
    f isa GB300Model || error("EnsembleGB300 needs an ODEFunction wrapping a GB300Model")
    model = MODEL_IDS[f.name]
    n = maximum(length(p.u0) for p in probs)
    npar = N_PARAMS[model]
    # C layout x[i*N + j] (trajectory fastest) is Julia's column-major (N, n) array
    u0 = zeros(N, n); ps = zeros(N, npar); ts = zeros(N, 2)
    for (j, p) in enumerate(probs)
        u0[j, 1:length(p.u0)] .= p.u0
        ps[j, :] .= p.p
        ts[j, 1], ts[j, 2] = p.tspan
    end
    npt = all(length(p.u0) == n for p in probs) ? C_NULL : Int32[length(p.u0) for p in probs]
    # saveat rules of lib/OrdinaryDiffEqCore/src/solve.jl:141-143,596-599,1103-1124
    scalar = saveat isa Number
    # (t0 + tdir|d|):(tdir|d|):tf; the library takes the points ascending in either direction
    t0, tf = probs[1].tspan
    sd = (tf < t0 ? -1 : 1) * abs(saveat isa Number ? saveat : 0.0)
    sv = scalar ? sort(collect(t0 + sd:sd:tf)) : sort(collect(Float64, saveat))
    ss = save_start === nothing ? (save_everystep || isempty(saveat) || scalar || probs[1].tspan[1] in sv) :
         save_start
    se = save_end === nothing ? (save_everystep || isempty(saveat) || scalar || probs[1].tspan[2] in sv) : save_end
    everystep = save_everystep   # with saveat too: both sets are kept (_savevalues!)
    callback === nothing || callback isa GB300Callback ||
        error("EnsembleGB300 runs the model's registered callback only: pass GB300Callback(...)")
    cb = callback isa GB300Callback
    # the solve's tstops (solve.jl:1021-1040): the library keeps those inside each (t0, tf)
    tst = collect(Float64, tstops)
    # save_idxs (1-based in Julia, 0-based in the library): the states kept, one row each
    sidx = save_idxs === nothing ? Int32[] : Int32[i - 1 for i in save_idxs]
    rows = save_idxs === nothing ? n : length(sidx)
    # a dt of either sign is taken in the direction of the span (handle_dt!, solve.jl:968-985)
    cg, ck, cqmax, cqmaxfirst = controller_knobs(controller)
    # isoutofdomain: the library runs the common (u, p, t) -> any(x -> x < 0, u), asked for by :negative
    isoutofdomain === nothing || isoutofdomain === :negative ||
        error("EnsembleGB300 runs isoutofdomain = :negative (any state < 0) only")
    iood = isoutofdomain === :negative ? Int32(1) : Int32(0)
    # array tolerances: one per state (the scalar fields then hold their smallest entries)
    atv = abstol isa AbstractVector ? collect(Float64, abstol) : Float64[]
    rtv = reltol isa AbstractVector ? collect(Float64, reltol) : Float64[]
    atol_s = isempty(atv) ? Float64(abstol) : minimum(atv)
    rtol_s = isempty(rtv) ? Float64(reltol) : minimum(rtv)
    o = Options(rtol_s, atol_s, dtmax, dtmin, abs(dt), maxiters, ss, se, save_end === nothing ? -1 : Int32(save_end),
                scalar, length(sv), 0, cqmaxfirst, cqmax, ens.lanes_per_traj, ens.scheduler, 0, -1, everystep,
                everystep ? max_step_saves : 0, cb, cb ? callback.interp_points : 10, cb ? callback.max_events : 0,
                length(tst), isempty(tst) ? Ptr{Float64}(C_NULL) : pointer(tst), jac_reuse(alg)[1], iood,
                jac_reuse(alg)[2], length(sidx), Int32(0), isempty(sidx) ? Ptr{Int32}(C_NULL) : pointer(sidx),
                Int32(adaptive), Int32(0), cg, Int32(force_dtmin), ck...,
                isempty(atv) ? Ptr{Float64}(C_NULL) : pointer(atv), isempty(rtv) ? Ptr{Float64}(C_NULL) : pointer(rtv))
    d = ProblemDesc(model, alg_id(alg), n, npar, ens.precision === :mixed ? 1 : 0, 0)
    cap = length(sv) + (everystep ? max_step_saves : 0) + 2 + (cb ? 2 * callback.max_events : 0)
    t_out = fill(NaN, N, cap); u_out = fill(NaN, N, rows, cap)   # [(s*rows + i)*N + j] -> u_out[j, i, s]
    nsaved = zeros(Int32, N); rc = zeros(Int32, N); st = Vector{Stats}(undef, N)
    # dense output (solve.jl:145-146) for every-step saves of one state count
    isdense = dense && everystep && npt == C_NULL && save_idxs === nothing
    GC.@preserve tst sidx atv rtv if isdense   # o holds pointers into tst, sidx, atv and rtv
        nk = ccall((:ode_dense_nk, LIB), Cint, (Cint,), alg_id(alg))
        k_out = zeros(N, n, nk, cap)   # [((s*nk + q)*n + i)*N + j] -> k_out[j, i, q, s]
        status = ccall((:ode_solve_ensemble_dense, LIB), Cint,
                       (Ptr{Cvoid}, Ref{ProblemDesc}, Ref{Options}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                        Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Int32}, Ptr{Stats}),
                       handle(ens.device), d, o, N, u0, ps, ts, t_out, u_out, k_out, nsaved, rc, st)
    else
        status = ccall((:ode_solve_ensemble, LIB), Cint,
                       (Ptr{Cvoid}, Ref{ProblemDesc}, Ref{Options}, Int64, Ptr{Int32}, Ptr{Float64}, Ptr{Float64},
                        Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Int32}, Ptr{Stats}),
                       handle(ens.device), d, o, N, npt, u0, ps, ts, sv, t_out, u_out, nsaved, rc, st)
    end
    status == 0 || error("ode_solve_ensemble: ", unsafe_string(ccall((:ode_last_error, LIB), Cstring, (Ptr{Cvoid},), handle(ens.device))))
    sols = map(1:N) do j
        k = nsaved[j]
        nj = save_idxs === nothing ? length(probs[j].u0) : rows
        us = [u_out[j, 1:nj, s] for s in 1:k]
        stats = SciMLBase.DEStats(st[j].nf, 0, 0, st[j].nsolve, st[j].nw, st[j].njacs, 0, 0, 0, 0,
                                  st[j].naccept, st[j].nreject, 0.0)
        if isdense
            interp = GB300DenseInterpolation(model, alg_id(alg), ps[j, :], ens.device, t_out[j, 1:k],
                                             u_out[j, :, 1:k], k_out[j, :, :, 1:k])
            SciMLBase.build_solution(probs[j], alg, t_out[j, 1:k], us; dense = true, interp,
                                     retcode = RETCODES[rc[j] + 1], stats)
        else
            SciMLBase.build_solution(probs[j], alg, t_out[j, 1:k], us; retcode = RETCODES[rc[j] + 1], stats)
        end
    end
    SciMLBase.EnsembleSolution(sols, time() - t0, true)
end

end # module
