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

using SparseArrays
import SmoothedParticles
import SmoothedParticles: create_cell_list!, apply!, apply_unary!, apply_binary!,
                          new_pvd_file, save_frame!, save_pvd_file, assemble_matrix,
                          assemble_vector

export GPUParticleSystem, DensitySum, ReferenceDensitySum, InternalForce, WallPressure,
       FindPressure, ResetRho, ResetRho0, ResetA, Accelerate, Move, Hydrostatic,
       upload!, download, upload_field!, particle_types, upload_ids, step!, init_state!,
       set_tuning!, memory_estimate, memory_usage, isidle, synchronize!, pair_count,
       GPUBatch, GPUVtkSeries, GPUMatrix, cg

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
    eos::Int32           # 0: Tait (P/rho^2 in the force), 1: linear c0^2 (rho - rho0) (P/rho0^2)
    cell_factor::Float64 # cell size / h: 0 or 1 (the reference's cells); 1..2 for mixed precision
end

abstract type BuiltinOperator end
struct DensitySum <: BuiltinOperator end          # find_rho!      -> SPH_OP_DENSITY
struct ReferenceDensitySum <: BuiltinOperator end # find_rho0!     -> SPH_OP_DENSITY_REF
struct InternalForce <: BuiltinOperator end       # internal_force! -> SPH_OP_FORCE
struct WallPressure <: BuiltinOperator end        # SPH_OP_WALL_PRESSURE
struct ResetRho <: BuiltinOperator end            # reset_rho!     -> SPH_OP_RESET_RHO
struct ResetRho0 <: BuiltinOperator end
struct ResetA <: BuiltinOperator end              # reset_a!
struct FindPressure <: BuiltinOperator end        # find_pressure! -> SPH_OP_EOS (the params' eos)
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

"ParticleField assignment: a whole field (:x, :v, :a, :xsph as 3 x n; :rho, :rho0,
:P as n; set :rho before :P) in sys.particles order."
function upload_field!(sys::GPUParticleSystem, var::Symbol, values::Array{Float64})
    id, comps = FIELDS[var]
    n = num_particles(sys)
    want = comps == 3 ? (3, n) : (n,)
    size(values) == want || throw(DimensionMismatch("$var: expected $want, got $(size(values))"))
    check(sys, ccall((:sph_set_field, libsphgpu), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                     sys.handle, id, values))
end

"Particle types (0 fluid, 1 wall) in sys.particles order."
function particle_types(sys::GPUParticleSystem)
    out = Vector{Int32}(undef, num_particles(sys))
    check(sys, ccall((:sph_get_field, libsphgpu), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                     sys.handle, 8, out))
    return out
end

"Each particle's index at upload time (1-based), in sys.particles order: what the
tail-fill removal of create_cell_list! (core.jl:57-70) did to the particle set."
function upload_ids(sys::GPUParticleSystem)
    out = Vector{Int64}(undef, num_particles(sys))
    check(sys, ccall((:sph_get_field, libsphgpu), Cint, (Ptr{Cvoid}, Cint, Ptr{Cvoid}),
                     sys.handle, 9, out))
    return out .+ 1
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

"""sum(sys, func, x) at the columns of a 3 x m matrix (2D points as well: z = 0);
func: 1 density, 2 kernel, 3 pressure, 4 Shepard."""
function SmoothedParticles.sum(sys::GPUParticleSystem, func::Integer, x::Matrix{Float64})
    # the library reads m points of 3 doubles each
    size(x, 1) == 3 || throw(DimensionMismatch(
        "query points must be a 3 x m matrix (got $(size(x, 1)) x $(size(x, 2)))"))
    out = Vector{Float64}(undef, size(x, 2))
    check(sys, ccall((:sph_sum_point, libsphgpu), Cint,
                     (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Ptr{Float64}),
                     sys.handle, func, size(x, 2), x, out))
    return out
end

"sum(sys, func, p) for the particles sys.particles[idx] (1-based indices)."
function SmoothedParticles.sum(sys::GPUParticleSystem, func::Integer,
                               idx::AbstractVector{<:Integer})
    index = Int64[i - 1 for i in idx]
    out = Vector{Float64}(undef, length(index))
    check(sys, ccall((:sph_sum_particle, libsphgpu), Cint,
                     (Ptr{Cvoid}, Cint, Int64, Ptr{Int64}, Ptr{Float64}),
                     sys.handle, func, length(index), index, out))
    return out
end

"Waits for the system's queued work; reports a device-side error as an exception."
synchronize!(sys::GPUParticleSystem) =
    check(sys, ccall((:sph_synchronize, libsphgpu), Cint, (Ptr{Cvoid},), sys.handle))

"Pair-interactions acted on since the last reset (the reference's action! calls)."
function pair_count(sys::GPUParticleSystem; reset::Bool = false)
    c = Ref{UInt64}(0)
    check(sys, ccall((:sph_pair_count, libsphgpu), Cint, (Ptr{Cvoid}, Ref{UInt64}, Cint),
                     sys.handle, c, reset))
    return Int(c[])
end

"verlet_step! of collapse_symplectic.jl, nsteps times, on the device (four or more
steps per call replay a captured two-step CUDA graph)."
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

# ---- ParaView export (IO.jl:15-75): the gather is queued on the system's
# stream, the copy and the .vtp write overlap the following steps

const FIELD_BITS = Dict(:x => 1, :v => 2, :a => 3, :xsph => 4, :rho => 5, :rho0 => 6, :P => 7,
                        :type => 8)

mutable struct GPUVtkSeries
    handle::Ptr{Cvoid}
    frames::Int
end

"new_pvd_file(path) (IO.jl:20-27) for a device system: frames <path>/frame<k>.vtp."
function new_pvd_file(sys::GPUParticleSystem, path::AbstractString)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(sys, ccall((:sph_vtk_open, libsphgpu), Cint, (Ptr{Cvoid}, Cstring, Ref{Ptr{Cvoid}}),
                     sys.handle, path, h))
    return GPUVtkSeries(h[], 0)
end

"save_frame!(data, sys, vars...) (IO.jl:53-63): positions plus the named fields."
function save_frame!(data::GPUVtkSeries, sys::GPUParticleSystem, vars::Symbol...)
    bits = UInt32(0)
    for v in vars
        bits |= UInt32(1) << FIELD_BITS[v]
    end
    k = Ref{Int32}(0)
    rc = ccall((:sph_vtk_save_frame, libsphgpu), Cint, (Ptr{Cvoid}, Cuint, Float64, Ref{Int32}),
               data.handle, bits, Float64(data.frames), k)
    rc == 0 || error("sph_vtk_save_frame failed ($rc)")
    data.frames = k[] + 1
    return nothing
end

"save_pvd_file(data) (IO.jl:33-35): waits for every frame and writes result.pvd."
function save_pvd_file(data::GPUVtkSeries)
    rc = ccall((:sph_vtk_close, libsphgpu), Cint, (Ptr{Cvoid},), data.handle)
    data.handle = C_NULL
    rc == 0 || error("sph_vtk_close: a frame or the collection could not be written ($rc)")
    return nothing
end

# ---- assemble_matrix / assemble_vector (core.jl:164-225) with the built-in
# functions: 1 the kernel W, 2 the ISPH projection matrix (param = C_free);
# the matrix stays on the device for cg

mutable struct GPUMatrix
    handle::Ptr{Cvoid}
    n::Int
    function GPUMatrix(h::Ptr{Cvoid})
        n, nnz = Ref{Int64}(0), Ref{Int64}(0)
        ccall((:sph_csr_info, libsphgpu), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}), h, n, nnz)
        a = new(h, Int(n[]))
        finalizer(x -> ccall((:sph_csr_destroy, libsphgpu), Cint, (Ptr{Cvoid},), x.handle), a)
        return a
    end
end

function assemble_matrix(sys::GPUParticleSystem, func::Integer, param::Real = 0.0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(sys, ccall((:sph_assemble_matrix, libsphgpu), Cint,
                     (Ptr{Cvoid}, Cint, Float64, Ref{Ptr{Cvoid}}), sys.handle, func, param, h))
    return GPUMatrix(h[])
end

"The matrix on the host as a SparseMatrixCSC (rows and columns in sys.particles order)."
function SparseArrays.sparse(a::GPUMatrix)
    n, nnz = Ref{Int64}(0), Ref{Int64}(0)
    ccall((:sph_csr_info, libsphgpu), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}), a.handle, n, nnz)
    rp = Vector{Int64}(undef, n[] + 1)
    col = Vector{Int32}(undef, nnz[])
    val = Vector{Float64}(undef, nnz[])
    rc = ccall((:sph_csr_download, libsphgpu), Cint,
               (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int32}, Ptr{Float64}), a.handle, rp, col, val)
    rc == 0 || error("sph_csr_download failed ($rc)")
    I = Vector{Int}(undef, nnz[])
    for r in 1:n[], k in (rp[r] + 1):rp[r + 1]
        I[k] = r
    end
    return sparse(I, Int.(col) .+ 1, val, n[], n[])
end

function assemble_vector(sys::GPUParticleSystem, func::Integer)
    out = Vector{Float64}(undef, num_particles(sys))
    check(sys, ccall((:sph_assemble_vector, libsphgpu), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}),
                     sys.handle, func, out))
    return out
end

"cg(A, b) of IterativeSolvers on the device (x0 = 0, until ||r|| <= reltol ||b||)."
function cg(a::GPUMatrix, b::Vector{Float64}; reltol::Real = sqrt(eps(Float64)),
            maxiter::Integer = -1)
    length(b) == a.n || throw(DimensionMismatch("b has $(length(b)) entries, A is $(a.n)"))
    x = Vector{Float64}(undef, a.n)
    it, res = Ref{Int32}(0), Ref{Float64}(0.0)
    rc = ccall((:sph_cg, libsphgpu), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64, Int32, Ref{Int32}, Ref{Float64}),
               a.handle, b, x, reltol, maxiter, it, res)
    rc == 0 || error("sph_cg failed ($rc)")
    return x
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

function synchronize!(b::GPUBatch)
    rc = ccall((:sph_batch_synchronize, libsphgpu), Cint, (Ptr{Cvoid},), b.handle)
    rc == 0 || error(unsafe_string(ccall((:sph_batch_last_error, libsphgpu), Cstring,
                                         (Ptr{Cvoid},), b.handle)))
    return nothing
end

end # module
