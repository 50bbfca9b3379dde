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
import ButterflyFactorizations
using ButterflyFactorizations: cluster_root, cluster_children, cluster_values, cluster_center,
                               cluster_radius, cluster_testtree, cluster_trialtree
import ButterflyFactorizations: PetrovGalerkinBF, assemble_BF, recompress_BF

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

# ---------------------------------------------------------------------------
# Construction on the GPU.  The reference's calls keep their signatures:
#   PetrovGalerkinBF(operator, testspace, trialspace, tree, k; tol, ...)
#       (src/Matrixassembly/petrovgalerkinbf.jl:33-54)
#   assemble_BF(kernelmatrix, blktree, no, ns, k, tau; ...)
#       (src/ButterflyFactorization/bfassembly.jl:48-62)
# with the point Helmholtz kernel G(r) = exp(-ikr)/(4 pi r) as the operator
# and 3 x N point matrices as the test / trial spaces.  The tree is any tree
# that implements the reference's tree interface (src/treeinterface.jl:39-164):
# it is converted once into the library's tree arrays.

"Point Helmholtz kernel exp(-ikr)/(4 pi r): the operator / kernel matrix of the GPU build."
struct HelmholtzPoints end

# bf_build_opts (include/bfgpu.h), field for field
struct BuildOpts
    c_tau::Float64
    min_samples::Int32
    adaptive::Int32
    seed::UInt64
    rank_mode::Int32
    keep_mixed::Int32
    surrogate_weights::Ptr{Float32}
    surrogate_nweights::Int64
    surrogate_margin::Float64
    factor_storage::Int32
    estimator::Int32      # 0: ButterflyRankEstimator(c_tau), 1: GeometricRankEstimator
    geo_rmin::Int32
    geo_c::Float64
    geo_ceps::Float64
end

const BF_STORE_C32 = Int32(0)
const BF_STORE_FF = Int32(1)

mutable struct GPUTree
    h::Ptr{Cvoid}
    order::Vector{Int}   # library node (0-based position + 1) -> reference node
end

"""
    GPUTree(tree, npoints) -> GPUTree

The library's tree arrays (bf_tree_from_arrays) from a tree with the reference
interface: nodes renumbered breadth first (children contiguous), points in
depth-first leaf order, so that every node's values are one contiguous range.
Half-sizes follow the TwoNTree relation radius = halfsize * sqrt(3)
(ext/BFH2Trees/BFH2Trees.jl:15-16).
"""
function GPUTree(tree, npoints::Integer)
    root = cluster_root(tree)
    order = [root]
    first = Int32[]; nchild = Int32[]; parent = Int32[-1]
    i = 1
    while i <= length(order)
        kids = collect(cluster_children(tree, order[i]))
        push!(first, isempty(kids) ? Int32(0) : Int32(length(order)))
        push!(nchild, Int32(length(kids)))
        for c in kids
            push!(order, c); push!(parent, Int32(i - 1))
        end
        i += 1
    end
    n = length(order)
    perm = Int64[]; bgn = zeros(Int64, n); en = zeros(Int64, n)
    function dfs(k)
        bgn[k] = length(perm)
        if nchild[k] == 0
            append!(perm, cluster_values(tree, order[k]) .- 1)
        else
            for c in 0:(nchild[k] - 1)
                dfs(first[k] + c + 1)
            end
        end
        en[k] = length(perm)
    end
    dfs(1)
    length(perm) == npoints || error("GPUTree: the leaves hold $(length(perm)) of $npoints points")
    center = Float64[]
    for nd in order
        append!(center, collect(cluster_center(tree, nd)))
    end
    half = [cluster_radius(tree, nd) / sqrt(3.0) for nd in order]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bf_tree_from_arrays, lib), Cint,
                (Int64, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32},
                 Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ref{Ptr{Cvoid}}),
                n, npoints, center, half, parent, first, nchild, bgn, en, perm, h),
          "bf_tree_from_arrays")
    t = GPUTree(h[], order)
    finalizer(x -> ccall((:bf_tree_destroy, lib), Cint, (Ptr{Cvoid},), x.h), t)
    return t
end

"""
    nearandfar_gpu(testtree, trialtree; alpha, minbflvl, leafcomp, leafimbalance,
                   unbalancedints, ctx=nothing)

Far pairs (library node ids, 0-based) and the near-pair count: the dual-tree
traversal of src/Matrixassembly/intlists.jl:30-217 with the AABB isFarFunctor
of ext/BFH2Trees/h2admissible.jl:11-45.  With `ctx` a Context the traversal
runs on that GPU (bf_nearandfar_gpu) and gives the same pairs in the same
order; without it, on the host (bf_nearandfar).
"""
function nearandfar_gpu(to::GPUTree, ts::GPUTree; alpha=1.0, minbflvl=3, leafcomp=true,
                        leafimbalance=true, unbalancedints=false, ctx=nothing)
    ctx === nothing || return _nearandfar_device(ctx, to, ts, alpha, minbflvl, leafcomp,
                                                 leafimbalance, unbalancedints)[1:3]
    nf = Ref{Int64}(0); nn = Ref{Int64}(0)
    args(fo, fs, cap) = ccall((:bf_nearandfar, lib), Cint,
                              (Ptr{Cvoid}, Ptr{Cvoid}, Float64, Int32, Int32, Int32, Int32,
                               Ptr{Int64}, Ptr{Int64}, Int64, Ref{Int64}, Ref{Int64}),
                              to.h, ts.h, alpha, minbflvl, leafcomp, leafimbalance,
                              unbalancedints, fo, fs, cap, nf, nn)
    check(args(C_NULL, C_NULL, 0), "bf_nearandfar")
    fo = zeros(Int64, max(nf[], 1)); fs = zeros(Int64, max(nf[], 1))
    check(args(fo, fs, length(fo)), "bf_nearandfar")
    return fo[1:nf[]], fs[1:nf[]], Int(nn[])
end

# one device traversal: far pairs, near-pair count, near pairs
function _nearandfar_device(ctx::Context, to::GPUTree, ts::GPUTree, alpha, minbflvl, leafcomp,
                            leafimbalance, unbalancedints)
    nf = Ref{Int64}(0); nn = Ref{Int64}(0)
    args(fo, fs, fcap, no, ns, ncap) =
        ccall((:bf_nearandfar_gpu, lib), Cint,
              (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Float64, Int32, Int32, Int32, Int32,
               Ptr{Int64}, Ptr{Int64}, Int64, Ptr{Int64}, Ptr{Int64}, Int64,
               Ref{Int64}, Ref{Int64}),
              ctx.h, to.h, ts.h, alpha, minbflvl, leafcomp, leafimbalance, unbalancedints,
              fo, fs, fcap, no, ns, ncap, nf, nn)
    check(args(C_NULL, C_NULL, 0, C_NULL, C_NULL, 0), "bf_nearandfar_gpu")
    fo = zeros(Int64, max(nf[], 1)); fs = zeros(Int64, max(nf[], 1))
    no = zeros(Int64, max(nn[], 1)); ns = zeros(Int64, max(nn[], 1))
    check(args(fo, fs, length(fo), no, ns, length(no)), "bf_nearandfar_gpu")
    return fo[1:nf[]], fs[1:nf[]], Int(nn[]), no[1:nn[]], ns[1:nn[]]
end

function _build(ctx::Context, X::AbstractMatrix{Float64}, Y::AbstractMatrix{Float64},
                to::GPUTree, ts::GPUTree, fo::Vector{Int64}, fs::Vector{Int64}, k, tol;
                c_tau, adaptive, seed, min_samples, storage, rankestimator=nothing)
    size(X, 1) == 3 && size(Y, 1) == 3 || error("point sets are 3 x N matrices")
    # the reference's estimator objects (rankestimation.jl:13-41) map onto the options
    est, gc, ge, gr = Int32(0), 1.5, 1.5, Int32(3)
    if rankestimator isa ButterflyFactorizations.GeometricRankEstimator
        est, gc, ge, gr = Int32(1), rankestimator.C, rankestimator.Cε, Int32(rankestimator.Rmin)
    elseif rankestimator isa ButterflyFactorizations.ButterflyRankEstimator
        c_tau = rankestimator.Cε
    end
    o = Ref(BuildOpts(c_tau, min_samples, adaptive, seed, 0, 1, C_NULL, 0, 0.15,
                      storage === :ff ? BF_STORE_FF : BF_STORE_C32, est, gr, gc, ge))
    x = Matrix{Float64}(X); y = Matrix{Float64}(Y)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bf_build, lib), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Cvoid}, Ptr{Cvoid},
                 Ptr{Int64}, Ptr{Int64}, Int64, Float64, Float64, Ref{BuildOpts},
                 Ref{Ptr{Cvoid}}),
                ctx.h, x, size(x, 2), y, size(y, 2), to.h, ts.h, fo, fs, length(fo), k, tol, o,
                h), "bf_build")
    return _wrap(h[])
end

"""
    near_pairs_gpu(testtree, trialtree; alpha, minbflvl, leafcomp, leafimbalance,
                   unbalancedints, ctx=nothing)

Near pairs (library node ids, 0-based) of the same traversal as nearandfar_gpu,
on the GPU of `ctx` when one is given.
"""
function near_pairs_gpu(to::GPUTree, ts::GPUTree; alpha=1.0, minbflvl=3, leafcomp=true,
                        leafimbalance=true, unbalancedints=false, ctx=nothing)
    ctx === nothing || return _nearandfar_device(ctx, to, ts, alpha, minbflvl, leafcomp,
                                                 leafimbalance, unbalancedints)[4:5]
    nn = Ref{Int64}(0)
    args(no, ns, cap) = ccall((:bf_near_pairs, lib), Cint,
                              (Ptr{Cvoid}, Ptr{Cvoid}, Float64, Int32, Int32, Int32, Int32,
                               Ptr{Int64}, Ptr{Int64}, Int64, Ref{Int64}),
                              to.h, ts.h, alpha, minbflvl, leafcomp, leafimbalance,
                              unbalancedints, no, ns, cap, nn)
    check(args(C_NULL, C_NULL, 0), "bf_near_pairs")
    no = zeros(Int64, max(nn[], 1)); ns = zeros(Int64, max(nn[], 1))
    check(args(no, ns, length(no)), "bf_near_pairs")
    return no[1:nn[]], ns[1:nn[]]
end

"""
    PetrovGalerkinBF(HelmholtzPoints(), X, Y, tree, k; tol=1e-3, alpha=1.0, Ctau=2.9592,
                     minbflvl=3, leafcomp=true, leafimbalance=true, unbalancedints=false,
                     adaptive=true, farfieldonly=false, storage=:c32, ctx=Context(0))

The reference's PetrovGalerkinBF (petrovgalerkinbf.jl:33-54) built on the GPU:
the trees of `tree` (cluster_testtree / cluster_trialtree) are converted, the
far pairs come from nearandfar_gpu and every far pair is compressed by
bf_build; unless `farfieldonly` (the reference's default is false) the near
blocks of the near pairs are evaluated on the GPU and attached
(bf_op_add_near), so that mul! gives near + far as in matrixvector.jl:28-33.
Returns a GPUButterflyOperator (a LinearMap).  `storage = :ff` keeps the far
factors as 16-byte float-float entries.
"""
function PetrovGalerkinBF(::HelmholtzPoints, X::AbstractMatrix{Float64},
                          Y::AbstractMatrix{Float64}, tree, k::Float64; tol=1e-3, alpha=1.0,
                          Ctau=2.9592, minbflvl=3, leafcomp=true, leafimbalance=true,
                          unbalancedints=false, adaptive=true, farfieldonly=false, seed=0,
                          min_samples=10, storage=:c32, rankestimator=nothing,
                          ctx::Context=Context(0))
    to = GPUTree(cluster_testtree(tree), size(X, 2))
    ts = GPUTree(cluster_trialtree(tree), size(Y, 2))
    fo, fs, _ = nearandfar_gpu(to, ts; alpha, minbflvl, leafcomp, leafimbalance, unbalancedints)
    A = _build(ctx, X, Y, to, ts, fo, fs, k, tol; c_tau=Ctau, adaptive=Int32(adaptive),
               seed=UInt64(seed), min_samples=Int32(min_samples), storage, rankestimator)
    if !farfieldonly
        no, ns = near_pairs_gpu(to, ts; alpha, minbflvl, leafcomp, leafimbalance, unbalancedints)
        x = Matrix{Float64}(X); y = Matrix{Float64}(Y)
        check(ccall((:bf_op_add_near, lib), Cint,
                    (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Float64}, Int64, Ptr{Cvoid},
                     Ptr{Cvoid}, Ptr{Int64}, Ptr{Int64}, Int64, Float64),
                    A.h, x, size(x, 2), y, size(y, 2), to.h, ts.h, no, ns, length(no), k),
              "bf_op_add_near")
    end
    return A
end

"""
    recompress_BF(A::GPUButterflyOperator, tau)

The reference's recompress_BF (src/Butterflyalgebra/algrecomp.jl:19-31) over
every far block of A, on the GPU (bf_op_recompress): a new operator, A is
unchanged.  A must hold the far field only.
"""
function recompress_BF(A::GPUButterflyOperator, tau::Real)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bf_op_recompress, lib), Cint, (Ptr{Cvoid}, Float64, Ref{Ptr{Cvoid}}),
                A.h, Float64(tau), h), "bf_op_recompress")
    return _wrap(h[])
end

"""
    adjoint_copy(A) / transpose_copy(A)

The reference's materialised adjoint(BF) / transpose(BF)
(src/Butterflyalgebra/bfadjtr.jl:43-67) over every far block
(bf_op_adjoint_copy): a new operator applied by the forward kernels.
"""
function _adjoint_copy(A::GPUButterflyOperator, trans::Integer)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bf_op_adjoint_copy, lib), Cint, (Ptr{Cvoid}, Cint, Ref{Ptr{Cvoid}}),
                A.h, Cint(trans), h), "bf_op_adjoint_copy")
    return _wrap(h[])
end
adjoint_copy(A::GPUButterflyOperator) = _adjoint_copy(A, 1)
transpose_copy(A::GPUButterflyOperator) = _adjoint_copy(A, 2)

"""
    save(A::GPUButterflyOperator, path) / load(ctx, path)

A built operator to a file and back (bf_op_save / bf_op_load): a second run
skips the construction.
"""
save(A::GPUButterflyOperator, path::AbstractString) =
    check(ccall((:bf_op_save, lib), Cint, (Ptr{Cvoid}, Cstring), A.h, path), "bf_op_save")
function load(ctx::Context, path::AbstractString)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:bf_op_load, lib), Cint, (Ptr{Cvoid}, Cstring, Ref{Ptr{Cvoid}}), ctx.h, path, h),
          "bf_op_load")
    return _wrap(h[])
end

"""
    assemble_BF(HelmholtzPoints(), blktree, no, ns, k, tau; X, Y, Ctau=4.0, adaptive=true,
                storage=:c32, ctx=Context(0))

One far block, as the reference's assemble_BF (bfassembly.jl:48-62): observer
node `no` of the test tree against source node `ns` of the trial tree (the
reference's 1-based node ids), compressed on the GPU.
"""
function assemble_BF(::HelmholtzPoints, blktree, no::Int, ns::Int, k::Float64, tau::Float64;
                     X::AbstractMatrix{Float64}, Y::AbstractMatrix{Float64}, Ctau=4.0,
                     adaptive=true, seed=0, min_samples=10, storage=:c32,
                     rankestimator=nothing, ctx::Context=Context(0))
    to = GPUTree(cluster_testtree(blktree), size(X, 2))
    ts = GPUTree(cluster_trialtree(blktree), size(Y, 2))
    fo = Int64[findfirst(==(no), to.order) - 1]
    fs = Int64[findfirst(==(ns), ts.order) - 1]
    return _build(ctx, X, Y, to, ts, fo, fs, k, tau; c_tau=Ctau, adaptive=Int32(adaptive),
                  seed=UInt64(seed), min_samples=Int32(min_samples), storage, rankestimator)
end

"""
    check(A::GPUButterflyOperator)

Raises if a bounded device-side wait of an asynchronous matvec on `A` gave up
since the last check (bf_op_check).
"""
check(A::GPUButterflyOperator) =
    check(ccall((:bf_op_check, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), A.h, C_NULL), "bf_op_check")

end # module
