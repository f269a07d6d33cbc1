# NPBAppsGPUChainRules.jl -- ChainRulesCore rule for NPBAppsGPU.terminal_objective:
# reverse mode through the GPU's hand-written discrete adjoint (npbmz_adjoint),
# checkpointing every `checkpoint_every` steps.  Include after NPBAppsGPU.jl in an
# environment that has ChainRulesCore:
#
#     include("NPBAppsGPU.jl"); include("NPBAppsGPUChainRules.jl")
#     J, back = Zygote.pullback(f -> NPBAppsGPU.terminal_objective(gpu, f, u0, ut, 50), forcing)
#
# The pullback's tangents for forcing and u0 are dJ/dforcing and dJ/du0 scaled by
# the incoming cotangent; the problem handle, the target and nsteps get none.
import ChainRulesCore

const CHECKPOINT_EVERY = Ref(10)

function ChainRulesCore.rrule(::typeof(NPBAppsGPU.terminal_objective), p::NPBAppsGPU.Problem,
                              forcing::Vector{Float64}, u0::Vector{Float64}, u_target::Vector{Float64},
                              nsteps::Integer)
    NPBAppsGPU.upload_all!(p, NPBAppsGPU.FORCING, forcing)
    NPBAppsGPU.upload_all!(p, NPBAppsGPU.U, u0)
    J, gf, gu = NPBAppsGPU.adjoint(p, nsteps, u_target; checkpoint_every = CHECKPOINT_EVERY[])
    function terminal_objective_pullback(dJ)
        s = ChainRulesCore.unthunk(dJ)
        return (ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent(), s .* gf, s .* gu,
                ChainRulesCore.NoTangent(), ChainRulesCore.NoTangent())
    end
    return J, terminal_objective_pullback
end
