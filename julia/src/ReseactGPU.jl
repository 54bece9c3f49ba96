# ReseactGPU.jl -- Julia binding of libreseact_gb300.so (include/reseact_gb300.h).
#
# The structs below are isbits mirrors of the C structs, so `ccall` passes them by
# reference exactly as the C ABI declares.  `lie_trotter_solve_bisect` keeps the keyword
# signature of OpSplit.lie_trotter_solve_bisect (tools/reactant_handoff/op_split.jl:219-241)
# so the call site at run_reseact.jl:350 changes by its first two arguments only.
# (Julia is not installed in the build container; this file is exercised through the same
# ABI by the Python ctypes tests.)
module ReseactGPU

const LIB = Ref{String}(get(ENV, "RESEACT_GB300_LIB",
    joinpath(@__DIR__, "..", "..", "reseact", "esm_gb300", "_build", "libreseact_gb300.so")))

const RS_OK = Int32(0)
const RS_ERR_MAXITERS = Int32(3)
const RS_ERR_NONFINITE = Int32(4)

struct RsMechanism
    n_species::Int32; n_reactions::Int32; n_params::Int32; combinatoric::Int32
    react_ptr::Ptr{Int32}; react_species::Ptr{Int32}; react_nu::Ptr{Int32}
    prod_ptr::Ptr{Int32}; prod_species::Ptr{Int32}; prod_coef::Ptr{Float64}
    prog_ptr::Ptr{Int32}; prog_op::Ptr{Int32}; prog_val::Ptr{Float64}
    params::Ptr{Float64}
end

struct RsGrid
    nlon::Int32; nlat::Int32; nlev::Int32; lon_bc::Int32; lat_bc::Int32
    lon0_deg::Float64; dlon_deg::Float64; lat0_deg::Float64; dlat_deg::Float64
end

struct RsController
    beta1::Float64; beta2::Float64; qmin::Float64; qmax::Float64; gamma::Float64
    qsteady_min::Float64; qsteady_max::Float64; qoldinit::Float64
end

struct RsConfig
    api_version::Int32; device::Int32; grid::RsGrid
    has_air_mass::Int32; do_transport::Int32; do_chemistry::Int32
    mech::RsMechanism
    rtol_T::Float64; atol_T::Float64; rtol_C::Float64; atol_C::Float64
    ctrl_T::RsController; ctrl_C::RsController
    maxiters::Float64; clamp_nonneg::Int32; precision::Int32; chem_mode::Int32
end

struct RsForcing
    mx::Ptr{Float64}; my::Ptr{Float64}; mz::Ptr{Float64}; flux_omega::Float64
    dp::Ptr{Float64}; qbc_w::Ptr{Float64}; qbc_e::Ptr{Float64}; qbc_s::Ptr{Float64}
    qbc_n::Ptr{Float64}; temperature::Ptr{Float64}; pressure::Ptr{Float64}
    emission::Ptr{Float64}
    pblh::Ptr{Float64}; ps::Ptr{Float64}; hyb_a::Ptr{Float64}; hyb_b::Ptr{Float64}
    tau_pblmix::Float64
    dps_dt::Ptr{Float64}
end

mutable struct RsStats
    naT::Float64; nrT::Float64; naC::Float64; nrC::Float64
    dtT_end::Float64; dtC_end::Float64; tT_end::Float64; tC_end::Float64
    chem_cell_steps::Float64; kernel_launches::Float64; status::Int32
end
RsStats() = RsStats(0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0)

mutable struct Handle
    ptr::Ptr{Cvoid}
    keep::Vector{Any}        # host arrays the structs point into (kept alive)
end

lasterr(h) = unsafe_string(ccall((:rs_last_error, LIB[]), Cstring, (Ptr{Cvoid},), h))

function check(h::Handle, rc::Int32)
    rc == RS_OK || error("reseact_gb300: ", lasterr(h.ptr), " (status $rc)")
    return nothing
end

"Create a solver handle (the arrays behind `mech` and `forcing` must stay alive)."
function create(cfg::RsConfig; keep = Any[])
    out = Ref{Ptr{Cvoid}}(C_NULL)
    rc = ccall((:rs_create, LIB[]), Int32, (Ref{RsConfig}, Ref{Ptr{Cvoid}}), cfg, out)
    rc == RS_OK || error("rs_create: ", lasterr(C_NULL), " (status $rc)")
    h = Handle(out[], keep)
    finalizer(h) do x
        x.ptr == C_NULL || ccall((:rs_destroy, LIB[]), Cvoid, (Ptr{Cvoid},), x.ptr)
        x.ptr = C_NULL
    end
    return h
end

set_forcing!(h::Handle, f::RsForcing) =
    check(h, ccall((:rs_set_forcing, LIB[]), Int32, (Ptr{Cvoid}, Ref{RsForcing}), h.ptr, f))

set_state!(h::Handle, u::Vector{Float64}) =
    check(h, ccall((:rs_set_state, LIB[]), Int32, (Ptr{Cvoid}, Ptr{Float64}, Csize_t),
                   h.ptr, u, length(u)))

function get_state!(h::Handle, u::Vector{Float64})
    check(h, ccall((:rs_get_state, LIB[]), Int32, (Ptr{Cvoid}, Ptr{Float64}, Csize_t),
                   h.ptr, u, length(u)))
    return u
end

"One Lie-Trotter macro step over [t0, t1] on the resident state (adv(...) analogue)."
function macro_step!(h::Handle, t0, t1, dtT, dtC)
    a = Ref(Float64(dtT)); b = Ref(Float64(dtC)); st = RsStats()
    rc = ccall((:rs_macro_step, LIB[]), Int32,
               (Ptr{Cvoid}, Float64, Float64, Ref{Float64}, Ref{Float64}, Ref{RsStats}),
               h.ptr, Float64(t0), Float64(t1), a, b, st)
    return rc, a[], b[], st
end

"""
    lie_trotter_solve(h, u0, tspan; macro_dt, dtT=15.0, dtC=0.5, refresh, forcing_tstops)

GPU version of OpSplit.lie_trotter_solve: same stop grid (macro-dt lattice joined with the
forcing boundaries in the half-open (t0, tf] and tf), same refresh rule, same return fields.
"""
function lie_trotter_solve(h::Handle, u0, tspan; macro_dt, dtT = 15.0, dtC = 0.5,
                           refresh = (_t -> nothing), forcing_tstops = Float64[],
                           clamp_nonneg::Bool = true)
    t0 = Float64(tspan[1]); tf = Float64(tspan[2])
    set_state!(h, collect(Float64, u0))
    fstops = Set(round(t; digits = 6) for t in forcing_tstops if t0 + 1e-6 < t <= tf + 1e-6)
    grid = collect((t0 + macro_dt):macro_dt:(tf - 1e-9))
    stops = sort!(unique!(vcat(grid, collect(fstops), Float64[tf])))
    tcur = t0; nmacro = 0; naT = nrT = naC = nrC = 0; retcode = :Success
    for tnext in stops
        tnext <= tcur + 1e-9 && continue
        rc, dtT, dtC, st = macro_step!(h, tcur, tnext, dtT, dtC)
        naT += Int(st.naT); nrT += Int(st.nrT); naC += Int(st.naC); nrC += Int(st.nrC)
        rc == RS_OK || (retcode = :Failure; break)
        tcur = tnext; nmacro += 1
        round(tcur; digits = 6) in fstops && refresh(tcur)
    end
    u = get_state!(h, similar(collect(Float64, u0)))
    return (; u, retcode, naT, nrT, naC, nrC, nmacro, dtT, dtC)
end

"Bisect-on-failure wrapper with the keyword signature of op_split.jl:219-241."
function lie_trotter_solve_bisect(h::Handle, u0, tspan; macro_dt, min_macro_dt::Real = 9.0,
                                  on_bisect = (_t0, _tf) -> nothing, kwargs...)
    t0 = Float64(tspan[1]); tf = Float64(tspan[2])
    r = lie_trotter_solve(h, u0, (t0, tf); macro_dt = macro_dt, kwargs...)
    (r.retcode == :Success || (tf - t0) <= min_macro_dt + 1e-9) && return r
    tm = 0.5 * (t0 + tf)
    on_bisect(t0, tf)
    r1 = lie_trotter_solve_bisect(h, u0, (t0, tm); macro_dt = min(Float64(macro_dt), tm - t0),
                                  min_macro_dt, on_bisect, kwargs...)
    r1.retcode == :Success || return r1
    kw2 = merge(NamedTuple(kwargs), (; dtT = r1.dtT, dtC = r1.dtC))
    r2 = lie_trotter_solve_bisect(h, r1.u, (tm, tf); macro_dt = min(Float64(macro_dt), tf - tm),
                                  min_macro_dt, on_bisect, kw2...)
    r2.retcode == :Success || return r2
    return (; u = r2.u, retcode = r2.retcode, naT = r1.naT + r2.naT, nrT = r1.nrT + r2.nrT,
            naC = r1.naC + r2.naC, nrC = r1.nrC + r2.nrC, nmacro = r1.nmacro + r2.nmacro,
            dtT = r2.dtT, dtC = r2.dtC)
end

# ---------------------------------------------------------------- the window solve in the library
struct RsSolveOpts
    macro_dt::Float64; min_macro_dt::Float64
    forcing_tstops::Ptr{Float64}; n_tstops::Csize_t
    refresh::Ptr{Cvoid}; on_bisect::Ptr{Cvoid}; user::Ptr{Cvoid}
end

mutable struct RsSolveResult
    naT::Float64; nrT::Float64; naC::Float64; nrC::Float64
    nmacro::Float64; nbisect::Float64; nrefresh::Float64; status::Int32; pad::Int32
end
RsSolveResult() = RsSolveResult(0, 0, 0, 0, 0, 0, 0, 0, 0)

# callbacks: the library passes back the `user` pointer, here the Julia context object
mutable struct SolveCtx
    refresh::Any
    on_bisect::Any
end
_refresh_tramp(user::Ptr{Cvoid}, t::Float64) =
    ((unsafe_pointer_to_objref(user)::SolveCtx).refresh(t); nothing)
_bisect_tramp(user::Ptr{Cvoid}, t0::Float64, t1::Float64) =
    ((unsafe_pointer_to_objref(user)::SolveCtx).on_bisect(t0, t1); nothing)

"""
    solve_window!(h, t0, t1; macro_dt, min_macro_dt=9.0, forcing_tstops, refresh, on_bisect,
                  dtT=15.0, dtC=0.5)

lie_trotter_solve_bisect done inside the library (rs_lie_trotter_solve) on the device-resident
state: the same stop grid, refresh rule and bisection, with the window's start state kept on
the GPU for a restart.  Returns (; retcode, naT, nrT, naC, nrC, nmacro, nbisect, dtT, dtC).
"""
function solve_window!(h::Handle, t0, t1; macro_dt, min_macro_dt::Real = 9.0,
                       forcing_tstops = Float64[], refresh = (_t -> nothing),
                       on_bisect = (_a, _b) -> nothing, dtT = 15.0, dtC = 0.5)
    ctx = SolveCtx(refresh, on_bisect)
    ts = collect(Float64, forcing_tstops)
    rf = @cfunction(_refresh_tramp, Cvoid, (Ptr{Cvoid}, Float64))
    bf = @cfunction(_bisect_tramp, Cvoid, (Ptr{Cvoid}, Float64, Float64))
    a = Ref(Float64(dtT)); b = Ref(Float64(dtC)); r = RsSolveResult()
    rc = GC.@preserve ctx ts begin
        opts = RsSolveOpts(Float64(macro_dt), Float64(min_macro_dt),
                           isempty(ts) ? C_NULL : pointer(ts), length(ts), rf, bf,
                           pointer_from_objref(ctx))
        ccall((:rs_lie_trotter_solve, LIB[]), Int32,
              (Ptr{Cvoid}, Float64, Float64, Ref{Float64}, Ref{Float64}, Ref{RsSolveOpts},
               Ref{RsSolveResult}), h.ptr, Float64(t0), Float64(t1), a, b, opts, r)
    end
    return (; retcode = rc == RS_OK ? :Success : :Failure, naT = Int(r.naT), nrT = Int(r.nrT),
            naC = Int(r.naC), nrC = Int(r.nrC), nmacro = Int(r.nmacro),
            nbisect = Int(r.nbisect), dtT = a[], dtC = b[])
end

# ---------------------------------------------------------------- discrete adjoint
record!(h::Handle, on::Bool) =
    check(h, ccall((:rs_record, LIB[]), Int32, (Ptr{Cvoid}, Int32), h.ptr, Int32(on)))
record_count(h::Handle) = Int(ccall((:rs_record_count, LIB[]), Int32, (Ptr{Cvoid},), h.ptr))
# device tape of the next recording: bytes, -1 = a quarter of free device memory, 0 = replay only
set_adjoint_tape!(h::Handle, budget_bytes::Integer) =
    check(h, ccall((:rs_set_adjoint_tape, LIB[]), Int32, (Ptr{Cvoid}, Int64), h.ptr,
                   Int64(budget_bytes)))
record_taped(h::Handle) = Int(ccall((:rs_record_taped, LIB[]), Int32, (Ptr{Cvoid},), h.ptr))
set_lambda!(h::Handle, lam::Vector{Float64}) =
    check(h, ccall((:rs_adjoint_set_lambda, LIB[]), Int32, (Ptr{Cvoid}, Ptr{Float64}, Csize_t),
                   h.ptr, lam, length(lam)))
function get_lambda!(h::Handle, lam::Vector{Float64})
    check(h, ccall((:rs_adjoint_get_lambda, LIB[]), Int32, (Ptr{Cvoid}, Ptr{Float64}, Csize_t),
                   h.ptr, lam, length(lam)))
    return lam
end
backward_macro_step!(h::Handle, k::Integer) =
    check(h, ccall((:rs_backward_macro_step, LIB[]), Int32, (Ptr{Cvoid}, Int32), h.ptr, Int32(k)))
"Frozen-dt replay of recorded macro step k on the resident state (replay_fixed)."
replay_macro_step!(h::Handle, k::Integer) =
    check(h, ccall((:rs_replay_macro_step, LIB[]), Int32, (Ptr{Cvoid}, Int32), h.ptr, Int32(k)))
function grad_emission!(h::Handle, g::Vector{Float64})
    check(h, ccall((:rs_adjoint_get_grad_emission, LIB[]), Int32,
                   (Ptr{Cvoid}, Ptr{Float64}, Csize_t), h.ptr, g, length(g)))
    return g
end
reset_grad!(h::Handle) = check(h, ccall((:rs_adjoint_reset_grad, LIB[]), Int32, (Ptr{Cvoid},), h.ptr))

"""
    forward_with_pullback(h, u0, tspan; macro_dt, kwargs...)

The windowed forward (lie_trotter_solve without bisection) recorded for the discrete adjoint,
and its pullback: ū_end -> (ū_0, ē) with ē the gradient w.r.t. the emission forcing, by the
library's backward sweep over the recorded macro steps (checkpoint + recomputation per step).
This is what the ChainRulesCore rrule of the package extension returns.
"""
function forward_with_pullback(h::Handle, u0, tspan; kwargs...)
    record!(h, true)
    r = lie_trotter_solve(h, u0, tspan; kwargs...)
    record!(h, false)
    r.retcode == :Success || error("forward window failed; nothing to differentiate")
    nrec = record_count(h)
    function pullback(ubar_end::AbstractVector)
        reset_grad!(h)
        set_lambda!(h, collect(Float64, ubar_end))
        for k in (nrec - 1):-1:0
            backward_macro_step!(h, k)
        end
        ubar0 = get_lambda!(h, similar(collect(Float64, ubar_end)))
        return ubar0
    end
    return r, pullback
end

# ---------------------------------------------------------------- kernel selection
const RS_CHEM_KERNEL_AUTO = Int32(0)
const RS_CHEM_KERNEL_TABLE = Int32(1)
const RS_CHEM_KERNEL_SPECIALIZED = Int32(2)
set_chem_kernel!(h::Handle, kind::Integer) =
    check(h, ccall((:rs_set_chem_kernel, LIB[]), Int32, (Ptr{Cvoid}, Int32), h.ptr, Int32(kind)))
function autotune!(h::Handle)
    buf = Vector{UInt8}(undef, 16384)
    check(h, ccall((:rs_autotune, LIB[]), Int32, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t),
                   h.ptr, buf, length(buf)))
    return unsafe_string(pointer(buf))
end
# replay launch shapes reported by an earlier autotune!, e.g.
# set_launch_shape!(h; xthreads=160, pencil=8, rows=32, yz_tracer_groups=6)
function set_launch_shape!(h::Handle; shapes...)
    for (k, v) in shapes
        check(h, ccall((:rs_set_launch_shape, LIB[]), Int32, (Ptr{Cvoid}, Cstring, Int32),
                       h.ptr, String(k), Int32(v)))
    end
    return h
end
const RS_STAGING_AUTO = Int32(0)
const RS_STAGING_PLAIN = Int32(1)
const RS_STAGING_BULK = Int32(2)
set_transport_staging!(h::Handle, mode::Integer) =
    check(h, ccall((:rs_set_transport_staging, LIB[]), Int32, (Ptr{Cvoid}, Int32), h.ptr, Int32(mode)))
function transport_staging(h::Handle)
    mode = Ref{Int32}(0)
    buf = Vector{UInt8}(undef, 512)
    check(h, ccall((:rs_get_transport_staging, LIB[]), Int32,
                   (Ptr{Cvoid}, Ref{Int32}, Ptr{UInt8}, Csize_t), h.ptr, mode, buf, length(buf)))
    return mode[], unsafe_string(pointer(buf))
end

end # module
