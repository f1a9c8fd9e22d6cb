# Julia binding of the GB300 HSS library (include/hssgpu.h) for HssMatrices.jl.
#
# A maintainer of HssMatrices.jl adds this module (or its methods) to route the
# hot path to the GPU: `mul!(C, hssA, B, a, b)` (src/matmul.jl:18),
# `hssA * B` (src/matmul.jl:13) and `hssA \ B` (src/hssmatrix.jl:234 ->
# `ulvfactsolve`, src/ulvfactor.jl:10), plus a resident factorization for
# repeated solves.  Every `ccall` signature here mirrors a prototype of
# include/hssgpu.h; tests/test_julia_shim.py checks them against the header.
module HssGpu

using HssMatrices, LinearAlgebra

const lib = joinpath(@__DIR__, "..", "lib", "libhssgpu.so")

const HSS_OK, HSS_ERR_BAD_DIMS, HSS_ERR_OOM, HSS_ERR_SINGULAR, HSS_ERR_NO_CONVERGENCE = 0, 1, 2, 3, 4
const HSS_ERR_TIMEOUT, HSS_ERR_CUDA, HSS_ERR_INVALID = 5, 6, 7
const FP64, FP32 = Int32(0), Int32(1)

struct SolveStats
    iterations::Int32
    converged::Int32
    residual::Float64
end

function check(rc)
    rc == HSS_OK && return
    msg = unsafe_string(ccall((:hss_last_error, lib), Cstring, ()))
    (rc == HSS_ERR_BAD_DIMS || rc == HSS_ERR_INVALID) && throw(DimensionMismatch(msg))
    rc == HSS_ERR_SINGULAR && throw(SingularException(0))
    rc == HSS_ERR_OOM && throw(OutOfMemoryError())
    error("hssgpu (status $rc): " * msg)
end

# pre-order walk: node table (16 Int64 per node) + packed generators
function pack(hssA::HssMatrix{Float64})
    rows = Vector{NTuple{16,Int64}}()
    buf = Float64[]
    put!(A) = isempty(A) ? -1 : (o = length(buf); append!(buf, vec(A)); o)
    function visit(h, isroot)
        i = length(rows)
        push!(rows, ntuple(_ -> 0, 16))
        if isleaf(h)
            ku, kv = isroot ? (0, 0) : (size(h.U, 2), size(h.V, 2))
            rows[i+1] = (-1, -1, size(h.D)..., ku, kv, put!(h.D),
                         isroot ? -1 : put!(h.U), isroot ? -1 : put!(h.V),
                         -1, -1, -1, -1, -1, -1, 0)
        else
            l = visit(h.A11, false)
            r = visit(h.A22, false)
            ku, kv = isroot ? (0, 0) : (size(h.R1, 2), size(h.W1, 2))
            rows[i+1] = (l, r, 0, 0, ku, kv, -1, -1, -1, put!(h.B12), put!(h.B21),
                         isroot ? -1 : put!(h.R1), isroot ? -1 : put!(h.R2),
                         isroot ? -1 : put!(h.W1), isroot ? -1 : put!(h.W2), 0)
        end
        return i
    end
    visit(hssA, true)
    table = [rows[i][f] for f in 1:16, i in 1:length(rows)]   # 16 x nnodes: node rows, column-major
    return table, buf
end

mutable struct GpuHss
    ptr::Ptr{Cvoid}
    m::Int
    n::Int
end

function GpuHss(hssA::HssMatrix{Float64})
    table, buf = pack(hssA)
    h = Ref{Ptr{Cvoid}}()
    check(ccall((:hss_create, lib), Cint, (Int64, Ptr{Int64}, Ptr{Float64}, Int64, Ref{Ptr{Cvoid}}),
                size(table, 2), table, buf, length(buf), h))
    g = GpuHss(h[], size(hssA)...)
    finalizer(x -> ccall((:hss_destroy, lib), Cint, (Ptr{Cvoid},), x.ptr), g)
end

# mul!(C, hssA, B, a, b) -- src/matmul.jl:18
function LinearAlgebra.mul!(C::Matrix{Float64}, g::GpuHss, B::Matrix{Float64}, a::Number, b::Number)
    check(ccall((:hss_matmul_host, lib), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Int64, Int64, Ptr{Float64}, Int64, Float64, Float64),
                g.ptr, B, stride(B, 2), size(B, 2), C, stride(C, 2), a, b))
    C
end
Base.:*(g::GpuHss, B::Matrix{Float64}) = mul!(zeros(g.m, size(B, 2)), g, B, 1.0, 0.0)
Base.:*(g::GpuHss, b::Vector{Float64}) = vec(g * reshape(b, :, 1))

# hssA \ B -- src/hssmatrix.jl:234 (FP32 ULV + FP64 refinement when prec == FP32)
function Base.:\(g::GpuHss, B::Matrix{Float64}; prec=FP64, tol=prec == FP32 ? 1e-10 : 0.0, maxit=10)
    X = zeros(g.n, size(B, 2))
    st = Ref{SolveStats}()
    check(ccall((:hss_ulvfactsolve_host, lib), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, Int64, Int64, Ptr{Float64}, Int64, Float64, Int32,
                 Ref{SolveStats}),
                g.ptr, prec, B, stride(B, 2), size(B, 2), X, stride(X, 2), tol, maxit, st))
    X
end
Base.:\(g::GpuHss, b::Vector{Float64}; kw...) = vec(\(g, reshape(b, :, 1); kw...))

# a resident factorization for repeated solves (new: the reference has only ulvfactsolve)
mutable struct GpuUlv
    ptr::Ptr{Cvoid}
    g::GpuHss
end

function ulvfactor(g::GpuHss; prec=FP64)
    f = Ref{Ptr{Cvoid}}()
    check(ccall((:hss_ulvfactor, lib), Cint, (Ptr{Cvoid}, Int32, Ref{Ptr{Cvoid}}, Ptr{Cvoid}),
                g.ptr, prec, f, C_NULL))
    F = GpuUlv(f[], g)
    finalizer(x -> ccall((:hss_factor_destroy, lib), Cint, (Ptr{Cvoid},), x.ptr), F)
end

function LinearAlgebra.ldiv!(X::Matrix{Float64}, F::GpuUlv, B::Matrix{Float64}; tol=0.0, maxit=10)
    st = Ref{SolveStats}()
    check(ccall((:hss_ulvsolve_host, lib), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Int64, Int64, Ptr{Float64}, Int64, Float64, Int32, Ref{SolveStats}),
                F.ptr, B, stride(B, 2), size(B, 2), X, stride(X, 2), tol, maxit, st))
    X
end

# a handle made on the device (division, adjoint), with its size
function adopt(h::Ptr{Cvoid})
    m, n = Ref{Int64}(), Ref{Int64}()
    check(ccall((:hss_size, lib), Cint, (Ptr{Cvoid}, Int32, Ref{Int64}, Ref{Int64}), h, Int32(0), m, n))
    g = GpuHss(h, m[], n[])
    finalizer(x -> ccall((:hss_destroy, lib), Cint, (Ptr{Cvoid},), x.ptr), g)
end

# hssA \ hssB and hssB / hssA -- src/ulvdivide.jl:13-17, src/hssmatrix.jl:235-237
function Base.:\(a::GpuHss, b::GpuHss; atol=1e-9, rtol=1e-9)
    h = Ref{Ptr{Cvoid}}()
    check(ccall((:hss_ldiv, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Float64, Float64, Ref{Ptr{Cvoid}}, Ptr{Cvoid}),
                a.ptr, b.ptr, atol, rtol, h, C_NULL))
    adopt(h[])
end
function Base.:/(b::GpuHss, a::GpuHss; atol=1e-9, rtol=1e-9)
    h = Ref{Ptr{Cvoid}}()
    check(ccall((:hss_rdiv, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Float64, Float64, Ref{Ptr{Cvoid}}, Ptr{Cvoid}),
                b.ptr, a.ptr, atol, rtol, h, C_NULL))
    adopt(h[])
end

# adjoint(hssA) -- src/hssmatrix.jl:165-171
function Base.adjoint(a::GpuHss)
    h = Ref{Ptr{Cvoid}}()
    check(ccall((:hss_transpose, lib), Cint, (Ptr{Cvoid}, Ref{Ptr{Cvoid}}, Ptr{Cvoid}), a.ptr, h, C_NULL))
    adopt(h[])
end

# refactor (after the generators changed) and solve in one call, the first
# solve's upward sweep pipelined behind the factorization (device buffers)
function factsolve!(X::Ptr{Float64}, ldx::Integer, F::GpuUlv, B::Ptr{Float64}, ldb::Integer, r::Integer;
                    tol=0.0, maxit=10, stream=C_NULL)
    st = Ref{SolveStats}()
    check(ccall((:hss_ulvfactsolve, lib), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Int64, Int64, Ptr{Float64}, Int64, Float64, Int32, Ref{SolveStats},
                 Ptr{Cvoid}),
                F.ptr, B, ldb, r, X, ldx, tol, maxit, st, stream))
    st[]
end

# process-wide switches (HSS_OPT_* of the header); HSS_OPT_GRAPHS = 4 also runs
# a refined solve's loop on the device (one graph, one status read per solve)
set_option(opt::Integer, value::Integer) =
    check(ccall((:hss_set_option, lib), Cint, (Int32, Int64), Int32(opt), Int64(value)))

# per-launch device times (ms, launch order) of one kernel kind (HSS_TRACE_* of
# the header) over the calls made between trace_begin and trace_times
trace_begin(kind::Integer) = check(ccall((:hss_trace_begin, lib), Cint, (Int32,), Int32(kind)))
function trace_times(cap::Integer=4096)
    ms = zeros(Float64, cap)
    n = Ref{Int64}(0)
    check(ccall((:hss_trace_times, lib), Cint, (Ptr{Float64}, Int64, Ref{Int64}), ms, cap, n))
    ms[1:min(n[], cap)]
end

end # module
