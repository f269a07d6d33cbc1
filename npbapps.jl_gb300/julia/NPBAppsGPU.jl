# NPBAppsGPU.jl -- Julia binding of libnpbmz_gpu.so (include/npbmz.h,
# include/npbmz_lu.h) for the NPBApps.jl BT-MZ / SP-MZ / LU-MZ node time loops.
#
# The reference's loop (src/BT/bt-node.jl:280-395, src/SP/sp-node.jl:252-397)
# calls exch_qbc(Val(ncells), ...) over all zones and then adi(iz, ...) per zone
# under Threads.@threads.  With this module the loop keeps its shape:
#
#     gpu = NPBAppsGPU.Problem(NPBAppsGPU.BT, nx, ny, nz, nbr, dt, gx, gy, gz, x_zones, y_zones)
#     NPBAppsGPU.setup!(gpu, ce)            # initialize + exact_rhs on the GPU
#     for STEP = 1:niter
#         NPBAppsGPU.exch_qbc!(gpu)          # replaces exch_qbc(...)
#         NPBAppsGPU.adi!(gpu)               # replaces the @threads adi(iz, ...) loop
#     end
#     xcr, xce = NPBAppsGPU.verify(gpu)      # replaces verify's node part
#
# or, where the Julia arrays must stay the source of truth each step,
# upload!/download! move one zone's OffsetArray (reference memory layout, halo
# untouched) in and out around the calls.  Every call checks the returned
# status and throws with npbmz_last_error's text; there is no CPU fallback.
module NPBAppsGPU

const libnpbmz = get(ENV, "NPBMZ_LIB", joinpath(@__DIR__, "..", "npbmz", "_build", "libnpbmz_gpu.so"))

const BT = Cint(0)
const SP = Cint(1)
const EXACT = Cint(0x1)
const MIXED = Cint(0x2)
const PERZONE = Cint(0x4)
const GRAPH = Cint(0x8)
const PERSIST = Cint(0x10)
const FP32_NOREFINE = Cint(0x20)
const REFINE_FP64 = Cint(0x40)
const RHS_DF = Cint(0x80)
const U = Cint(0)
const RHS = Cint(1)
const FORCING = Cint(2)
const LAYOUT_DENSE = Cint(0)
const LAYOUT_REF = Cint(1)

mutable struct Problem
    handle::Ptr{Cvoid}
    kind::Cint
    nzones::Int
    lock::ReentrantLock          # serialises calls on the handle (adi from Threads.@threads)
    function Problem(kind, nx::Vector{<:Integer}, ny, nz, nbr, dt, gx, gy, gz, x_zones, y_zones; flags = Cint(0))
        n = length(nx)
        # nbr: 4 per zone (west, east, south, north), 0-based zone numbers
        params = Cdouble[dt, gx, gy, gz, x_zones, y_zones]
        out = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:npbmz_create, libnpbmz), Cint,
                   (Cint, Cint, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Cdouble}, Cint, Ptr{Ptr{Cvoid}}),
                   kind, n, Cint.(nx), Cint.(ny), Cint.(nz), Cint.(nbr), params, flags, out)
        rc == 0 || error("npbmz_create: " * unsafe_string(ccall((:npbmz_last_error, libnpbmz), Cstring, (Ptr{Cvoid},), C_NULL)))
        p = new(out[], Cint(kind), n, ReentrantLock())
        finalizer(p) do q
            q.handle != C_NULL && ccall((:npbmz_destroy, libnpbmz), Cint, (Ptr{Cvoid},), q.handle)
            q.handle = C_NULL
        end
        return p
    end
end

check(p::Problem, rc, what) =
    rc == 0 || error(what * ": " * unsafe_string(ccall((:npbmz_last_error, libnpbmz), Cstring, (Ptr{Cvoid},), p.handle)))

"""Zone geometry of zone_setup (src/BT/zone_setup.jl); 0-based neighbours."""
function zone_setup(kind, gx, gy, gz, x_zones, y_zones, ratio)
    n = x_zones * y_zones
    nx = zeros(Cint, n); ny = zeros(Cint, n); nz = zeros(Cint, n); nbr = zeros(Cint, 4n)
    rc = ccall((:npbmz_zone_setup, libnpbmz), Cint,
               (Cint, Cint, Cint, Cint, Cint, Cint, Cdouble, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}),
               kind, gx, gy, gz, x_zones, y_zones, ratio, nx, ny, nz, nbr)
    rc == 0 || error("npbmz_zone_setup failed")
    return nx, ny, nz, nbr
end

"""initialize + exact_rhs on the GPU; ce is the reference's 5x13 table (set_constants.jl:47-51)."""
function setup!(p::Problem, ce::AbstractMatrix{Float64})
    c = Matrix{Float64}(permutedims(ce))      # the C side reads row-major [5][13]
    check(p, ccall((:npbmz_setup, libnpbmz), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.handle, c), "npbmz_setup")
end

"""Replaces exch_qbc(Val(ncells), ...) (src/BT/exchange_qbc.jl:1-122)."""
exch_qbc!(p::Problem) = check(p, ccall((:npbmz_exch_qbc, libnpbmz), Cint, (Ptr{Cvoid},), p.handle), "npbmz_exch_qbc")

"""Replaces adi(iz, ...) (src/BT/adi.jl:5-251): zone iz (1-based), or all zones batched."""
adi!(p::Problem, iz::Integer = 0) =
    check(p, ccall((:npbmz_adi, libnpbmz), Cint, (Ptr{Cvoid}, Cint), p.handle, iz - 1), "npbmz_adi")

"""Faces exchanged with zones of other MPI ranks (exch_qbc_send / exch_qbc_recv,
src/BT/exchange_qbc.jl:145-465): `send` and `recv` are vectors of (zone,
side) pairs, 1-based zones of this handle and sides 0..3 = west, east,
south, north, each received side marked NPBMZ_REMOTE (-1) in the nbr table
the handle was created with.  Returns the Float64 counts of the send and
receive buffers."""
function face_plan!(p::Problem, send::AbstractVector, recv::AbstractVector)
    flat(v) = Cint[x for (z, s) in v for x in (z - 1, s)]
    s = flat(send); r = flat(recv)
    ns = Ref{Int64}(0); nr = Ref{Int64}(0)
    check(p, ccall((:npbmz_face_plan, libnpbmz), Cint,
                   (Ptr{Cvoid}, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Ref{Int64}, Ref{Int64}),
                   p.handle, length(send), s, length(recv), r, ns, nr), "npbmz_face_plan")
    return ns[], nr[]
end

"""Pack the registered send faces into a device buffer (CuPtr or raw address)."""
pack_faces!(p::Problem, send_buf) =
    check(p, ccall((:npbmz_pack_faces, libnpbmz), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.handle, send_buf),
          "npbmz_pack_faces")

"""Unpack the registered receive faces from a device buffer into u's ghost planes."""
unpack_faces!(p::Problem, recv_buf) =
    check(p, ccall((:npbmz_unpack_faces, libnpbmz), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.handle, recv_buf),
          "npbmz_unpack_faces")

"""niter steps of exch_qbc + adi; returns the per-step (xcr, xce) norms when norms = true."""
function step!(p::Problem, niter::Integer; norms = false)
    if norms
        out = zeros(Cdouble, 10, niter)
        check(p, ccall((:npbmz_step, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}), p.handle, niter, out), "npbmz_step")
        return out
    end
    check(p, ccall((:npbmz_step, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}), p.handle, niter, C_NULL), "npbmz_step")
    return nothing
end

"""Choose the launch configuration (lines per CTA, zone-group branches of the
step graph, persistent kernels) by timing whole steps on the problem's own
data; u, rhs and forcing are left as they were and results do not change."""
function autotune!(p::Problem)
    check(p, ccall((:npbmz_autotune, libnpbmz), Cint, (Ptr{Cvoid},), p.handle), "npbmz_autotune")
    return nothing
end

"""verify's node part (src/BT/verify.jl:411-505): (xcr, xce) summed over zones."""
function verify(p::Problem)
    xcr = zeros(Cdouble, 5); xce = zeros(Cdouble, 5)
    check(p, ccall((:npbmz_verify, libnpbmz), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}), p.handle, xcr, xce), "npbmz_verify")
    return xcr, xce
end

"""Upload one zone's array in the reference's own OffsetArray memory
(u[z], rhs[z] or forcing[z] of bt_data.jl / sp_data.jl): pass the OffsetArray."""
upload!(p::Problem, zone::Integer, field, a) =
    check(p, ccall((:npbmz_upload, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Cdouble}),
                   p.handle, zone - 1, field, LAYOUT_REF, parent(a)), "npbmz_upload")

download!(p::Problem, zone::Integer, field, a) =
    check(p, ccall((:npbmz_download, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Cdouble}),
                   p.handle, zone - 1, field, LAYOUT_REF, parent(a)), "npbmz_download")

# ---- all zones at once, dense layout (zone z: [5][nz][ny][nx] row-major, i.e. a
# Julia Array{Float64}(undef, nx, ny, nz, 5) per zone, zones back to back) ----
upload_all!(p::Problem, field, x::Vector{Float64}) =
    check(p, ccall((:npbmz_upload, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Cdouble}),
                   p.handle, -1, field, LAYOUT_DENSE, x), "npbmz_upload")

function download_all(p::Problem, field, n::Integer)
    x = Vector{Float64}(undef, n)
    check(p, ccall((:npbmz_download, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Cdouble}),
                   p.handle, -1, field, LAYOUT_DENSE, x), "npbmz_download")
    return x
end

"""
    adjoint(p, nsteps, u_target; checkpoint_every = 10) -> (J, dJ/dforcing, dJ/du0)

Discrete adjoint of `nsteps` BT-MZ steps from the handle's current u and
forcing for J = 1/2 sum (u_N - u_target)^2 over every stored point
(npbmz_adjoint).  Dense all-zone vectors; u is left as it was.
"""
function adjoint(p::Problem, nsteps::Integer, u_target::Vector{Float64}; checkpoint_every::Integer = 10)
    n = length(u_target)
    J = Ref{Cdouble}(0.0)
    gf = Vector{Float64}(undef, n)
    gu = Vector{Float64}(undef, n)
    check(p, ccall((:npbmz_adjoint, libnpbmz), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Ptr{Cdouble}, Ref{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                   p.handle, nsteps, checkpoint_every, u_target, J, gf, gu), "npbmz_adjoint")
    return J[], gf, gu
end

"""
    terminal_objective(p, forcing, u0, u_target, nsteps) -> J

J = 1/2 sum (u_N - u_target)^2 after `nsteps` steps of exch_qbc + adi from
(u0, forcing), all dense all-zone vectors.  Differentiable through the rrule
in NPBAppsGPUChainRules.jl (the hand-written discrete adjoint on the GPU).
"""
function terminal_objective(p::Problem, forcing::Vector{Float64}, u0::Vector{Float64}, u_target::Vector{Float64},
                            nsteps::Integer)
    upload_all!(p, FORCING, forcing)
    upload_all!(p, U, u0)
    step!(p, nsteps)
    a = download_all(p, U, length(u0)) .- u_target
    upload_all!(p, U, u0)
    return 0.5 * sum(abs2, a)
end

"""
One zone's field held on the GPU.  Vectors of these stand in for the
reference's per-zone arrays u, rhs, forcing in its node loop, so that its own
adi / exch_qbc calls reach the GPU methods of NPBAppsGPUShim.jl.
"""
struct DeviceZone
    p::Problem
    zone::Int        # 1-based
    field::Cint
end

device_zones(p::Problem, field) = [DeviceZone(p, iz, Cint(field)) for iz in 1:p.nzones]

"""adi of one zone under the handle's lock (the reference calls adi from Threads.@threads)."""
adi_locked!(p::Problem, iz::Integer) = lock(() -> adi!(p, iz), p.lock)

# ---------------------------------------------------------------------------
# LU-MZ (include/npbmz_lu.h).  The reference's LU loop (src/LU/lu-node.jl:
# 233-270) keeps its shape:
#
#     lu = NPBAppsGPU.LuProblem(nx, ny, nz, nbr, dt)     # nbr from lu_zone_setup
#     NPBAppsGPU.setup!(lu)                              # setbv, setiv, erhs, rhs
#     for istep = 1:itmax
#         NPBAppsGPU.exch_qbc!(lu)                       # replaces exch_qbc(...)
#         NPBAppsGPU.ssor!(lu)                           # replaces the @threads ssor(iz, ...) loop
#     end
#     xcr, xce, xci = NPBAppsGPU.verify(lu)              # ERROR, l2norm, pintgr summed over zones

const LU_FACES_NPB = Cint(0x1)
const LU_GRAPH = Cint(0x2)
const LU_U = Cint(0)
const LU_RSD = Cint(1)
const LU_FRCT = Cint(2)

mutable struct LuProblem
    handle::Ptr{Cvoid}
    nzones::Int
    lock::ReentrantLock          # serialises calls on the handle (ssor from Threads.@threads)
    function LuProblem(nx::Vector{<:Integer}, ny, nz, nbr, dt; omega = 1.2, flags = Cint(0))
        n = length(nx)
        params = Cdouble[dt, omega]
        out = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:npbmz_lu_create, libnpbmz), Cint,
                   (Cint, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Cdouble}, Cint, Ptr{Ptr{Cvoid}}),
                   n, Cint.(nx), Cint.(ny), Cint.(nz), Cint.(nbr), params, flags, out)
        rc == 0 || error("npbmz_lu_create: " * unsafe_string(ccall((:npbmz_lu_last_error, libnpbmz), Cstring, (Ptr{Cvoid},), C_NULL)))
        p = new(out[], n, ReentrantLock())
        finalizer(p) do q
            q.handle != C_NULL && ccall((:npbmz_lu_destroy, libnpbmz), Cint, (Ptr{Cvoid},), q.handle)
            q.handle = C_NULL
        end
        return p
    end
end

check(p::LuProblem, rc, what) =
    rc == 0 || error(what * ": " * unsafe_string(ccall((:npbmz_lu_last_error, libnpbmz), Cstring, (Ptr{Cvoid},), p.handle)))

"""Zone sizes and LU's neighbours (src/LU/zone_setup.jl); 0-based neighbours."""
function lu_zone_setup(gx, gy, gz, x_zones, y_zones, ratio = 1.0)
    n = x_zones * y_zones
    nx = zeros(Cint, n); ny = zeros(Cint, n); nz = zeros(Cint, n); nbr = zeros(Cint, 4n)
    rc = ccall((:npbmz_lu_zone_setup, libnpbmz), Cint,
               (Cint, Cint, Cint, Cint, Cint, Cdouble, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}, Ptr{Cint}),
               gx, gy, gz, x_zones, y_zones, ratio, nx, ny, nz, nbr)
    rc == 0 || error("npbmz_lu_zone_setup: " * unsafe_string(ccall((:npbmz_lu_last_error, libnpbmz), Cstring, (Ptr{Cvoid},), C_NULL)))
    return nx, ny, nz, nbr
end

"""setbv, setiv, erhs and rhs on the GPU; ce = nothing: the reference's table (setcoeff.jl)."""
function setup!(p::LuProblem, ce::Union{Nothing, AbstractMatrix{Float64}} = nothing)
    c = ce === nothing ? Ptr{Cdouble}(C_NULL) : Matrix{Float64}(permutedims(ce))
    check(p, ccall((:npbmz_lu_setup, libnpbmz), Cint, (Ptr{Cvoid}, Ptr{Cdouble}), p.handle, c), "npbmz_lu_setup")
end

"""Replaces exch_qbc(...) (src/LU/exchange_qbc.jl)."""
exch_qbc!(p::LuProblem) =
    check(p, ccall((:npbmz_lu_exch_qbc, libnpbmz), Cint, (Ptr{Cvoid},), p.handle), "npbmz_lu_exch_qbc")

"""Replaces ssor(iz, ...) (src/LU/ssor.jl:9-254): zone iz (1-based), or all zones batched."""
ssor!(p::LuProblem, iz::Integer = 0) =
    check(p, ccall((:npbmz_lu_ssor, libnpbmz), Cint, (Ptr{Cvoid}, Cint), p.handle, iz - 1), "npbmz_lu_ssor")

"""niter iterations of exch_qbc + ssor; the per-iteration rsd norms when norms = true."""
function iterate!(p::LuProblem, niter::Integer; norms = false)
    out = norms ? zeros(Cdouble, 5, niter) : nothing
    check(p, ccall((:npbmz_lu_iterate, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Ptr{Cdouble}), p.handle, niter,
                   norms ? out : Ptr{Cdouble}(C_NULL)), "npbmz_lu_iterate")
    return out
end

"""ERROR, l2norm and pintgr summed over zones (src/LU/lu-node.jl:306-321): (xcr, xce, xci)."""
function verify(p::LuProblem)
    xcr = zeros(Cdouble, 5); xce = zeros(Cdouble, 5); xci = zeros(Cdouble, 1)
    check(p, ccall((:npbmz_lu_verify, libnpbmz), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
                   p.handle, xcr, xce, xci), "npbmz_lu_verify")
    return xcr, xce, xci[1]
end

"""One zone's u, rsd or frct in the reference's OffsetArray memory ([1:5, -1:nx+2, -1:ny+2, 1:nz])."""
upload!(p::LuProblem, zone::Integer, field, a) =
    check(p, ccall((:npbmz_lu_upload, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Cdouble}),
                   p.handle, zone - 1, field, LAYOUT_REF, parent(a)), "npbmz_lu_upload")
download!(p::LuProblem, zone::Integer, field, a) =
    check(p, ccall((:npbmz_lu_download, libnpbmz), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Cdouble}),
                   p.handle, zone - 1, field, LAYOUT_REF, parent(a)), "npbmz_lu_download")

"""One zone's u, rsd or frct of an LuProblem: vectors of these stand in for
the reference's u, rsd, frct in its LU loop (NPBAppsGPUShim.jl)."""
struct LuDeviceZone
    p::LuProblem
    zone::Int        # 1-based
    field::Cint
end

device_zones(p::LuProblem, field) = [LuDeviceZone(p, iz, Cint(field)) for iz in 1:p.nzones]

"""ssor of one zone under the handle's lock (the reference calls ssor from Threads.@threads)."""
ssor_locked!(p::LuProblem, iz::Integer) = lock(() -> ssor!(p, iz), p.lock)

end # module
