# BFGPU.jl -- Julia binding of libbfgpu.so (the C ABI in include/bfgpu.h).
#
# A package extension for ButterflyFactorizations.jl would include this file.
# It keeps the reference's operator interface: a LinearMap whose mul!/adjoint/
# transpose call the GPU, an importer for ButterflyFactorization objects built
# by assemble_BF (the parity path), and a GPU builder for the far field.
# Julia is not installed in the build image, so this file is not exercised by
# the test-suite; the same C ABI is exercised from Python (bfgpu/).
module BFGPU

using LinearAlgebra
using LinearMaps

const lib = get(ENV, "BFGPU_LIB", joinpath(@__DIR__, "..", "bfgpu", "libbfgpu.so"))

const BF_OP_N = Cint(0)
const BF_OP_C = Cint(1)
const BF_OP_T = Cint(2)
const BF_PTR_HOST = Cint(0)

lasterror() = unsafe_string(ccall((:bf_last_error, lib), Cstring, ()))
check(s::Cint, what) = s == 0 || error("$what failed: ", lasterror())

struct Context
    h::Ptr{Cvoid}
end
function Context(device::Integer=0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bf_ctx_create, lib), Cint, (Cint, Ref{Ptr{Cvoid}}), device, r), "bf_ctx_create")
    return Context(r[])
end

mutable struct GPUButterflyOperator <: LinearMaps.LinearMap{ComplexF64}
    h::Ptr{Cvoid}
    dims::Tuple{Int,Int}
    trans::Cint
    owner::Any
end

function _wrap(h::Ptr{Cvoid})
    r = Ref{Int64}(0); c = Ref{Int64}(0)
    check(ccall((:bf_op_size, lib), Cint, (Ptr{Cvoid}, Ref{Int64}, Ref{Int64}), h, r, c), "bf_op_size")
    op = GPUButterflyOperator(h, (Int(r[]), Int(c[])), BF_OP_N, nothing)
    finalizer(o -> ccall((:bf_op_destroy, lib), Cint, (Ptr{Cvoid},), o.h), op)
    return op
end

Base.size(A::GPUButterflyOperator) = A.trans == BF_OP_N ? A.dims : reverse(A.dims)

# adjoint(A) / transpose(A): lazy views on the same device factors
# (the reference materialises a copy, src/Butterflyalgebra/bfadjtr.jl:43-67)
LinearAlgebra.adjoint(A::GPUButterflyOperator) =
    GPUButterflyOperator(A.h, A.dims, A.trans == BF_OP_N ? BF_OP_C : BF_OP_N, A)
LinearAlgebra.transpose(A::GPUButterflyOperator) =
    GPUButterflyOperator(A.h, A.dims, A.trans == BF_OP_N ? BF_OP_T : BF_OP_N, A)

# mul!(y, A, x, α, β): y = β y + α op(A) x (src/matrixalgebra/matrixvector.jl:8-65)
function LinearAlgebra.mul!(y::StridedVecOrMat{ComplexF64}, A::GPUButterflyOperator,
                            x::StridedVecOrMat{ComplexF64}, α::Number, β::Number)
    a = ComplexF64[α]; b = ComplexF64[β]
    nrhs = size(x, 2)
    check(ccall((:bf_matvec, lib), Cint,
                (Ptr{Cvoid}, Cint, Int64, Ptr{ComplexF64}, Int64, Ptr{ComplexF64}, Int64,
                 Ptr{ComplexF64}, Ptr{ComplexF64}, Cint, Ptr{Cvoid}),
                A.h, A.trans, nrhs, x, max(stride(x, 2), size(x, 1)), y,
                max(stride(y, 2), size(y, 1)), a, b, BF_PTR_HOST, C_NULL), "bf_matvec")
    return y
end
LinearAlgebra.mul!(y::StridedVecOrMat{ComplexF64}, A::GPUButterflyOperator,
                   x::StridedVecOrMat{ComplexF64}) = mul!(y, A, x, true, false)
LinearMaps._unsafe_mul!(y, A::GPUButterflyOperator, x::AbstractVector) = mul!(y, A, x)

"""
    import_factors(ctx, bfs, testtree, trialtree, nrows, ncols) -> GPUButterflyOperator

Upload `ButterflyFactorization`s built by `assemble_BF` (bfstructs.jl:21-146). Keys and
cluster values are converted to 0-based; `UniformScaling` blocks become identity flags.
"""
function import_factors(ctx::Context, bfs, testtree, trialtree, nrows::Integer, ncols::Integer,
                        cluster_values, nnodes_test::Integer, nnodes_trial::Integer)
    bfid = Int32[]; stage = Int32[]; oo = Int64[]; so = Int64[]; oi = Int64[]; si = Int64[]
    rows = Int32[]; cols = Int32[]; ident = Int8[]; off = Int64[]; data = ComplexF64[]
    function push(i, st, b)
        push!(bfid, i - 1); push!(stage, st)
        push!(oo, b.obs_out - 1); push!(so, b.src_out - 1); push!(oi, b.obs_in - 1); push!(si, b.src_in - 1)
        push!(off, length(data))
        if b.data isa UniformScaling
            push!(rows, 0); push!(cols, 0); push!(ident, 1)
        else
            push!(rows, size(b.data, 1)); push!(cols, size(b.data, 2)); push!(ident, 0)
            append!(data, vec(b.data))
        end
    end
    for (i, bf) in enumerate(bfs)
        foreach(b -> push(i, 0, b), bf.Q)
        for (l, lvl) in enumerate(bf.R), b in lvl.blocks
            push(i, l, b)
        end
        foreach(b -> push(i, -1, b), bf.P)
    end
    csr(tree, nn) = begin
        ptr = Int64[0]; idx = Int64[]
        for node in 1:nn
            append!(idx, cluster_values(tree, node) .- 1); push!(ptr, length(idx))
        end
        ptr, idx
    end
    optr, oidx = csr(testtree, nnodes_test)
    sptr, sidx = csr(trialtree, nnodes_trial)
    desc = (Int64(nrows), Int64(ncols), Int64(length(bfid)), pointer(bfid), pointer(stage),
            pointer(oo), pointer(so), pointer(oi), pointer(si), pointer(rows), pointer(cols),
            pointer(ident), pointer(off), Ptr{Float64}(pointer(data)), Int64(nnodes_test),
            pointer(optr), pointer(oidx), Int64(nnodes_trial), pointer(sptr), pointer(sidx))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve bfid stage oo so oi si rows cols ident off data optr oidx sptr sidx begin
        d = Ref(desc)
        check(ccall((:bf_import_factors, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ref{Ptr{Cvoid}}),
                    ctx.h, Base.unsafe_convert(Ptr{Cvoid}, d), h), "bf_import_factors")
    end
    return _wrap(h[])
end

end # module
