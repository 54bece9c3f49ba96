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
    joinpath(@__DIR__, "..", "reseact", "esm_gb300", "_build", "libreseact_gb300.so")))

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

end # module
