# NPBAppsGPUShim.jl -- methods of the reference's own adi and exch_qbc for zones
# held on the GPU, so that the node loops of NPBApps.jl run unchanged.
#
#     include("NPBAppsGPU.jl"); include("NPBAppsGPUShim.jl")
#     gpu = NPBAppsGPU.Problem(...); NPBAppsGPU.setup!(gpu, ce)
#     u       = NPBAppsGPU.device_zones(gpu, NPBAppsGPU.U)
#     rhs     = NPBAppsGPU.device_zones(gpu, NPBAppsGPU.RHS)
#     forcing = NPBAppsGPU.device_zones(gpu, NPBAppsGPU.FORCING)
#
# and the loop of src/BT/bt-node.jl:280-395 (src/SP/sp-node.jl:252-397) passes
# these vectors where it passed its OffsetArrays.  Each method has the
# reference function's arity and types only the zone-array positions, so
# Julia dispatch prefers it exactly when those arguments are DeviceZones; the
# other arguments (MPI buffers, scratch, constants) are ignored: the library
# holds its own.  Positions: BT adi forcing / u / rhs at 14 / 15 / 16 of 76
# (src/BT/adi.jl:5-80); SP adi u / rhs at 11 / 12 and forcing at 26 of 99,
# after speed at 25 (src/SP/adi.jl:6-104, called so from
# src/SP/sp-node.jl:291-316); exch_qbc u at 17 of 25
# (src/BT/exchange_qbc.jl:1-26, src/SP/exchange_qbc.jl:1-26).  adi of one
# zone runs under the handle's lock, as the reference calls it from
# Threads.@threads; NPBAppsGPU.adi!(gpu) (all
# zones batched in one launch per phase) is the fast form of the same loop.
# The same for LU-MZ's ssor and exch_qbc (below).  Julia is not installed
# where this was written: unexecuted.
import NPBApps
using .NPBAppsGPU: DeviceZone, LuDeviceZone

function NPBApps.BT.adi(iz, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13,
                        forcing::DeviceZone, u::DeviceZone, rhs::DeviceZone, rest::Vararg{Any,60})
    NPBAppsGPU.adi_locked!(u.p, u.zone)
    return nothing
end

function NPBApps.SP.adi(z, a2, a3, a4, a5, a6, a7, a8, a9, a10, u::DeviceZone, rhs::DeviceZone,
                        a13, a14, a15, a16, a17, a18, a19, a20, a21, a22, a23, a24, a25,
                        forcing::DeviceZone, rest::Vararg{Any,73})
    NPBAppsGPU.adi_locked!(u.p, u.zone)
    return nothing
end

for M in (NPBApps.BT, NPBApps.SP)
    @eval function $M.exch_qbc(v::Val, a2, a3, a4, a5, a6, a7, a8, a9, a10, a11, a12, a13, a14, a15, a16,
                               u::AbstractVector{DeviceZone}, rest::Vararg{Any,8})
        p = u[1].p
        lock(() -> NPBAppsGPU.exch_qbc!(p), p.lock)
        return nothing
    end
end

# LU-MZ: ssor u / rsd / frct at 6 / 7 / 8 of 41 (src/LU/ssor.jl:9-50); exch_qbc
# u at 4 of 36 (src/LU/exchange_qbc.jl:17).  Pass
# NPBAppsGPU.device_zones(lu, NPBAppsGPU.LU_U) (LU_RSD, LU_FRCT) where
# src/LU/lu-node.jl:233-270 passes u, rsd, frct.
function NPBApps.LU.ssor(iz, ipt, jpt, proc_num_zones, comm_solve, u::LuDeviceZone, rsd::LuDeviceZone,
                         frct::LuDeviceZone, rest::Vararg{Any,33})
    NPBAppsGPU.ssor_locked!(u.p, u.zone)
    return nothing
end

function NPBApps.LU.exch_qbc(proc_num_zones, zone_proc_id, proc_zone_id, u::AbstractVector{LuDeviceZone},
                             rest::Vararg{Any,32})
    p = u[1].p
    lock(() -> NPBAppsGPU.exch_qbc!(p), p.lock)
    return nothing
end
