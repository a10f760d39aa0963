#=
SmoothedParticlesGPU.jl -- Julia binding of libsphgpu.so (include/sphgpu.h).

Keeps SmoothedParticles.jl's surface for the cell list and pair loop:
create_cell_list!, apply!, apply_unary!, apply_binary!, SmoothedParticles.sum,
dispatching on a GPUParticleSystem and on singleton types for the built-in
operators (arbitrary closures have no device counterpart; nothing runs on the
CPU).  Particle fields are moved as whole arrays in sys.particles order.

Untested here: no Julia runtime exists on the build or GPU machines.  The same
C ABI is exercised from Python (sphgpu/_lib.py) by the test suite.
=#
module SmoothedParticlesGPU

import SmoothedParticles
import SmoothedParticles: create_cell_list!, apply!, apply_unary!, apply_binary!

export GPUParticleSystem, DensitySum, ReferenceDensitySum, InternalForce, WallPressure,
       FindPressure, ResetRho, ResetRho0, ResetA, Accelerate, Move, Hydrostatic,
       upload!, download, step!, init_state!, set_tuning!, memory_estimate, memory_usage,
       isidle, GPUBatch

const libsphgpu = get(ENV, "SPHGPU_LIB", joinpath(@__DIR__, "..", "libsphgpu.so"))

struct SphParams
    dim::Int32
    precision::Int32
    h::Float64
    domain_min::NTuple{3,Float64}
    domain_max::NTuple{3,Float64}
    mass::Float64
    rho0::Float64
    c0::Float64
    h_smooth::Float64
    alpha::Float64
    eps_xsph::Float64
    gravity::NTuple{3,Float64}
    dt::Float64
    col_height::Float64
    vertical_axis::Int32
    reserved::Int32
end

abstract type BuiltinOperator end
struct DensitySum <: BuiltinOperator end          # find_rho!      -> SPH_OP_DENSITY
struct ReferenceDensitySum <: BuiltinOperator end # find_rho0!     -> SPH_OP_DENSITY_REF
struct InternalForce <: BuiltinOperator end       # internal_force! -> SPH_OP_FORCE
struct WallPressure <: BuiltinOperator end        # SPH_OP_WALL_PRESSURE
struct ResetRho <: BuiltinOperator end            # reset_rho!     -> SPH_OP_RESET_RHO
struct ResetRho0 <: BuiltinOperator end
struct ResetA <: BuiltinOperator end              # reset_a!
struct FindPressure <: BuiltinOperator end        # find_pressure! -> SPH_OP_EOS (Tait)
struct Accelerate <: BuiltinOperator end          # accelerate!    -> SPH_OP_KICK
struct Move <: BuiltinOperator end                # move!          -> SPH_OP_DRIFT
struct Hydrostatic <: BuiltinOperator end

opcode(::DensitySum) = 1
opcode(::ReferenceDensitySum) = 2
opcode(::InternalForce) = 3
opcode(::WallPressure) = 4
opcode(::ResetRho) = 10
opcode(::ResetRho0) = 11
opcode(::ResetA) = 12
opcode(::FindPressure) = 13
opcode(::Accelerate) = 14
opcode(::Move) = 15
opcode(::Hydrostatic) = 16
isbinary(op::BuiltinOperator) = opcode(op) <= 4

mutable struct GPUParticleSystem
    handle::Ptr{Cvoid}
    params::SphParams
    function GPUParticleSystem(p::SphParams; device::Integer = 0)
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:sph_create, libsphgpu), Cint, (Ref{SphParams}, Cint, Ref{Ptr{Cvoid}}),
                   p, device, h)
        rc == 0 || error("sph_create failed ($rc)")
        sys = new(h[], p)
        finalizer(s -> ccall((:sph_destroy, libsphgpu), Cint, (Ptr{Cvoid},), s.handle), sys)
        return sys
    end
end

function check(sys::GPUParticleSystem, rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:sph_last_error, libsphgpu), Cstring, (Ptr{Cvoid},), sys.handle))
    error("sphgpu error $rc: $msg")
end

"generate_particles! equivalent: x, v are 3 x n matrices; type 0 fluid, 1 wall."
function upload!(sys::GPUParticleSystem, x::Matrix{Float64}, v::Matrix{Float64},
                 type::Vector{Int32})
    n = size(x, 2)
    check(sys, ccall((:sph_upload, libsphgpu), Cint,
                     (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                      Ptr{Int32}), sys.handle, n, x, v, C_NULL, C_NULL, type))
end

function num_particles(sys::GPUParticleSystem)
    n = Ref{Int64}(0)
    check(sys, ccall((:sph_num_particles, libsphgpu), Cint, (Ptr{Cvoid}, Ref{Int64}),
                     sys.handle, n))
    return n[]
end

const FIELDS = Dict(:x => (1, 3), :v => (2, 3), :a => (3, 3), :xsph => (4, 3), :rho => (5, 1),
                    :rho0 => (6, 1), :P => (7, 1))

"ParticleField equivalent: the whole field in sys.particles order."
function download(sys::GPUParticleSystem, var::Symbol)
    id, comps = FIELDS[var]
    n = num_particles(sys)
    out = comps == 3 ? Matrix{Float64}(undef, 3, n) : Vector{Float64}(undef, n)
    check(sys, ccall((:sph_get_field, libsphgpu), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                     sys.handle, id, out))
    return out
end

create_cell_list!(sys::GPUParticleSystem) =
    check(sys, ccall((:sph_create_cell_list, libsphgpu), Cint, (Ptr{Cvoid},), sys.handle))

function apply!(sys::GPUParticleSystem, op::BuiltinOperator; self::Bool = false)
    if isbinary(op)
        check(sys, ccall((:sph_apply, libsphgpu), Cint, (Ptr{Cvoid}, Cint, Cint),
                         sys.handle, opcode(op), self))
    else
        apply_unary!(sys, op)
    end
end

apply_binary!(sys::GPUParticleSystem, op::BuiltinOperator) = apply!(sys, op; self = false)

apply_unary!(sys::GPUParticleSystem, op::BuiltinOperator) =
    check(sys, ccall((:sph_apply_unary, libsphgpu), Cint, (Ptr{Cvoid}, Cint),
                     sys.handle, opcode(op)))

"sum(sys, func, x) at the columns of a 3 x m matrix; func: 1 density, 2 kernel, 3 pressure, 4 Shepard."
function SmoothedParticles.sum(sys::GPUParticleSystem, func::Integer, x::Matrix{Float64})
    out = Vector{Float64}(undef, size(x, 2))
    check(sys, ccall((:sph_sum_point, libsphgpu), Cint,
                     (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Ptr{Float64}),
                     sys.handle, func, size(x, 2), x, out))
    return out
end

"verlet_step! of collapse_symplectic.jl, nsteps times, on the device."
step!(sys::GPUParticleSystem, nsteps::Integer = 1) =
    check(sys, ccall((:sph_step, libsphgpu), Cint, (Ptr{Cvoid}, Cint), sys.handle, nsteps))

init_state!(sys::GPUParticleSystem) =
    check(sys, ccall((:sph_init_state, libsphgpu), Cint, (Ptr{Cvoid},), sys.handle))

"Warps per block of the pair passes (2, 4 or 8); results do not depend on it."
set_tuning!(sys::GPUParticleSystem, warps::Integer) =
    check(sys, ccall((:sph_set_tuning, libsphgpu), Cint, (Ptr{Cvoid}, Cint), sys.handle, warps))

"Device bytes a system with parameters p holds with n particles (no GPU call)."
function memory_estimate(p::SphParams, n::Integer)
    b = Ref{UInt64}(0)
    rc = ccall((:sph_memory_estimate, libsphgpu), Cint, (Ref{SphParams}, Int64, Ref{UInt64}),
               p, n, b)
    rc == 0 || error("sph_memory_estimate failed ($rc)")
    return Int(b[])
end

function memory_usage(sys::GPUParticleSystem)
    b = Ref{UInt64}(0)
    check(sys, ccall((:sph_memory_usage, libsphgpu), Cint, (Ptr{Cvoid}, Ref{UInt64}),
                     sys.handle, b))
    return Int(b[])
end

"True when all work queued on the system's stream has finished (never waits)."
function isidle(sys::GPUParticleSystem)
    i = Ref{Cint}(0)
    check(sys, ccall((:sph_query, libsphgpu), Cint, (Ptr{Cvoid}, Ref{Cint}), sys.handle, i))
    return i[] == 1
end

"""
Many independent systems stepped together: every pair of steps is one CUDA-graph
launch in which each member is an independent branch.  Members must outlive the
batch; their results equal stepping each alone.
"""
mutable struct GPUBatch
    handle::Ptr{Cvoid}
    members::Vector{GPUParticleSystem}
    function GPUBatch(members::Vector{GPUParticleSystem})
        hs = [m.handle for m in members]
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:sph_batch_create, libsphgpu), Cint, (Ptr{Ptr{Cvoid}}, Cint, Ref{Ptr{Cvoid}}),
                   hs, length(hs), h)
        rc == 0 || error("sph_batch_create failed ($rc)")
        b = new(h[], members)
        finalizer(x -> ccall((:sph_batch_destroy, libsphgpu), Cint, (Ptr{Cvoid},), x.handle), b)
        return b
    end
end

function step!(b::GPUBatch, nsteps::Integer = 2)
    rc = ccall((:sph_batch_step, libsphgpu), Cint, (Ptr{Cvoid}, Cint), b.handle, nsteps)
    rc == 0 || error(unsafe_string(ccall((:sph_batch_last_error, libsphgpu), Cstring,
                                         (Ptr{Cvoid},), b.handle)))
    return nothing
end

end # module
