# ReseactGPUChainRulesExt.jl -- ChainRulesCore rule for the GPU windowed solve: the package
# extension that Project.toml declares ([weakdeps] ChainRulesCore, [extensions]), loaded
# when ChainRulesCore is present in the environment (Julia >= 1.9).  The pullback is the
# library's discrete adjoint: exact for the recorded accepted step sequence of both halves (the
# fixed-sequence VJP of rx_traced_integrator.jl:610-623 and adjoint_gradient.jl:731-835), with
# per-macro-step checkpoints and recomputation on the device.
module ReseactGPUChainRulesExt

using ChainRulesCore
using ReseactGPU: Handle, forward_with_pullback, lie_trotter_solve

function ChainRulesCore.rrule(::typeof(lie_trotter_solve), h::Handle, u0, tspan; kwargs...)
    r, back = forward_with_pullback(h, u0, tspan; kwargs...)
    function lie_trotter_solve_pullback(rbar)
        ubar_end = rbar.u isa ChainRulesCore.AbstractZero ? zero(r.u) : collect(rbar.u)
        return (NoTangent(), NoTangent(), back(ubar_end), NoTangent())
    end
    return r, lie_trotter_solve_pullback
end

end # module
