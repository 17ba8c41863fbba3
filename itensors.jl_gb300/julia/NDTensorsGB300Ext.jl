# NDTensorsGB300Ext: drop-in NDTensors storage backend calling libndtensors_gb300.so.
#
# Mirrors how NDTensors/ext/NDTensorsCUDAExt and NDTensors/ext/NDTensorscuTENSORExt
# plug into NDTensors through `Expose` dispatch: a device vector type `GB300Vector`
# is the data of Dense / BlockSparse storage, and the hot-path methods are
# overloaded for `Exposed{<:GB300Vector}`:
#
#   contract!(R, labelsR, T1, labelsT1, T2, labelsT2, α, β)      (NDTensors/ext/NDTensorscuTENSORExt/contract.jl:15-58)
#   permutedims!(R, T, perm)                                      (NDTensors/ext/NDTensorsCUDAExt/permutedims.jl:4-23)
#   contract(::BlockSparseTensor, ...) via contract_blockoffsets /
#   contract! with the plan built on the device                   (NDTensors/src/blocksparse/contract.jl:3-76)
#   svd(::BlockSparseMatrix)                                      (NDTensors/src/blocksparse/linearalgebra.jl:45-215)
#   qr(::BlockSparseMatrix) through qx                            (NDTensors/src/blocksparse/linearalgebra.jl:351-415)
#   truncate!!(::Type{<:GB300Vector}, P)                          (NDTensors/src/truncate.jl:15-20)
#   rrule(contract, T1, labels1, T2, labels2, labelsR) on block-sparse
#   storage, and the pullback contract_pullback_gb300 that
#   rrule(contract, ::ITensor, ::ITensor) hands GB300 storage to  (ext/ITensorsChainRulesCoreExt/itensor.jl:94-103)
#   contract(::BlockSparseTensor, ::DiagBlockSparseTensor)         (NDTensors/src/blocksparse/diagblocksparse.jl:601-696)
#   eigen(::Hermitian{<:BlockSparseMatrix})                       (NDTensors/src/blocksparse/linearalgebra.jl:221-348)
#   dot / norm / rmul! / axpby! on the storage vector, as reached by
#   inner / norm / scale! / add!                                  (ext/ITensorsVectorInterfaceExt/ITensorsVectorInterfaceExt.jl:5-84)
#
# Fermionic sign fixes of the reference's svd (right_arrow_sign / left_arrow_sign) are
# not applied: auto-fermion is off by default and this backend is bosonic (real FP64).
# Status: written against the C ABI in include/ndtensors_gb300.h; it has not been
# run (no Julia toolchain was available where this library was built and tested).
module NDTensorsGB300Ext

using NDTensors
using NDTensors: BlockSparseTensor, DenseTensor, Tensor, inds, data, blockoffsets, nzblocks,
    BlockOffsets, Block, blockdim, contract_labels
using NDTensors.Expose: Exposed, unexpose, expose
using NDTensors: DiagBlockSparseTensor, Spectrum, ind, dag, sim, setblock!, block, resize
using LinearAlgebra
using ChainRulesCore: ChainRulesCore, NoTangent

const LIB = get(ENV, "NDTENSORS_GB300_LIB", joinpath(@__DIR__, "..", "ndtensors_gb300", "libndtensors_gb300.so"))

const ND_ERR_NOCONV = Int32(3)
const ND_PREC_FP64 = Int32(0)
const ND_PREC_OZAKI = Int32(1)
const ND_PREC_BF16X3 = Int32(2)
const PRECISION = Ref(ND_PREC_FP64)          # drop-in default: plain FP64
set_precision!(p::Symbol) = (PRECISION[] = p === :ozaki ? ND_PREC_OZAKI : p === :bf16x3 ? ND_PREC_BF16X3 : ND_PREC_FP64)

struct NDError <: Exception
  status::Int32
  msg::String
end

const HANDLE = Ref{Ptr{Cvoid}}(C_NULL)
function handle()
  if HANDLE[] == C_NULL
    h = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:nd_create, LIB), Int32, (Int32, Ref{Ptr{Cvoid}}), 0, h)
    st == 0 || throw(NDError(st, unsafe_string(ccall((:nd_last_error, LIB), Cstring, (Ptr{Cvoid},), C_NULL))))
    HANDLE[] = h[]
  end
  return HANDLE[]
end

check(st) = st == 0 ? nothing :
  throw(NDError(st, unsafe_string(ccall((:nd_last_error, LIB), Cstring, (Ptr{Cvoid},), handle()))))

# Verify mode: split-precision contractions are recomputed in FP64 and the relative
# Frobenius distance of the last one is kept (0 for FP64 calls, -1 before any).
set_verify!(on::Bool) = check(ccall((:nd_set_verify, LIB), Int32, (Ptr{Cvoid}, Int32), handle(), on ? 1 : 0))
function verify_last()
  e = Ref{Float64}(-1.0)
  check(ccall((:nd_verify_last, LIB), Int32, (Ptr{Cvoid}, Ref{Float64}), handle(), e))
  return e[]
end

# ---- device vector --------------------------------------------------------
mutable struct GB300Vector <: AbstractVector{Float64}
  ptr::Ptr{Float64}
  len::Int
  function GB300Vector(::UndefInitializer, n::Integer)
    p = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:nd_alloc, LIB), Int32, (Ptr{Cvoid}, Csize_t, Ref{Ptr{Cvoid}}), handle(), max(n, 1) * 8, p))
    v = new(Ptr{Float64}(p[]), n)
    finalizer(x -> ccall((:nd_free, LIB), Int32, (Ptr{Cvoid}, Ptr{Cvoid}), handle(), x.ptr), v)
    return v
  end
end
Base.size(v::GB300Vector) = (v.len,)
Base.getindex(::GB300Vector, ::Int) = error("scalar indexing of a GB300Vector: copy to the host with Array(v)")
function Base.Array(v::GB300Vector)
  a = Vector{Float64}(undef, v.len)
  check(ccall((:nd_d2h, LIB), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), handle(), a, v.ptr, v.len * 8))
  return a
end
function gb300(a::AbstractVector{Float64})
  v = GB300Vector(undef, length(a))
  check(ccall((:nd_h2d, LIB), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), handle(), v.ptr, collect(a), length(a) * 8))
  return v
end

# a view of the first n elements that shares (and keeps alive) the parent's memory
mutable struct GB300View <: AbstractVector{Float64}
  parent::GB300Vector
  ptr::Ptr{Float64}
  len::Int
end
Base.size(v::GB300View) = (v.len,)
Base.getindex(::GB300View, ::Int) = error("scalar indexing of a GB300View: copy to the host with Array(v)")
function Base.Array(v::GB300View)
  a = Vector{Float64}(undef, v.len)
  check(ccall((:nd_d2h, LIB), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Csize_t), handle(), a, v.ptr, v.len * 8))
  return a
end

# ---- dense ----------------------------------------------------------------
function NDTensors.contract!(R::Exposed{<:GB300Vector,<:DenseTensor}, labelsR,
                             T1::Exposed{<:GB300Vector,<:DenseTensor}, labelsT1,
                             T2::Exposed{<:GB300Vector,<:DenseTensor}, labelsT2, α::Number=1.0, β::Number=0.0)
  r, t1, t2 = unexpose(R), unexpose(T1), unexpose(T2)
  dR, d1, d2 = Int64[size(r)...], Int64[size(t1)...], Int64[size(t2)...]
  check(ccall((:nd_contract_dense_f64, LIB), Int32,
              (Ptr{Cvoid}, Ptr{Float64}, Int32, Ptr{Int64}, Ptr{Int32}, Ptr{Float64}, Int32, Ptr{Int64}, Ptr{Int32},
               Ptr{Float64}, Int32, Ptr{Int64}, Ptr{Int32}, Float64, Float64, Int32),
              handle(), data(r).ptr, length(dR), dR, Int32[labelsR...], data(t1).ptr, length(d1), d1, Int32[labelsT1...],
              data(t2).ptr, length(d2), d2, Int32[labelsT2...], Float64(α), Float64(β), PRECISION[]))
  return r
end

function Base.permutedims!(R::Exposed{<:GB300Vector}, T::Exposed{<:GB300Vector}, perm)
  r, t = unexpose(R), unexpose(T)
  dT = Int64[size(t)...]
  check(ccall((:nd_permutedims_f64, LIB), Int32,
              (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Int32, Ptr{Int64}, Ptr{Int32}, Float64, Float64),
              handle(), data(r).ptr, data(t).ptr, length(dT), dT, Int32[perm...], 1.0, 0.0))
  return r
end

# ---- block sparse ---------------------------------------------------------
struct BsDesc
  rank::Int32
  nblocks::Ptr{Int32}
  blockdims::Ptr{Int64}
  nnzblocks::Int32
  blocks::Ptr{Int32}
  offsets::Ptr{Int64}
end

function desc_arrays(T::Union{BlockSparseTensor,DiagBlockSparseTensor})
  is = inds(T)
  nb = Int32[NDTensors.nblocks(i) for i in is]
  bd = Int64[NDTensors.blockdim(i, b) for i in is for b in 1:NDTensors.nblocks(i)]
  bofs = blockoffsets(T)
  blocks = Int32[]
  offs = Int64[]
  for (b, o) in pairs(bofs)
    append!(blocks, Int32.(Tuple(b)))
    push!(offs, o)
  end
  return nb, bd, blocks, offs, length(offs)
end

# The plan (block pairs, output blocks and offsets) is built on the device and
# is bit-exact with contract_blockoffsets(::Algorithm"sequential", ...).
function NDTensors.contract(T1::BlockSparseTensor{Float64,N1,<:NDTensors.BlockSparse{Float64,<:GB300Vector}}, labels1,
                            T2::BlockSparseTensor{Float64,N2,<:NDTensors.BlockSparse{Float64,<:GB300Vector}}, labels2,
                            labelsR=contract_labels(labels1, labels2)) where {N1,N2}
  plan = Ref(bs_plan(T1, labels1, T2, labels2, labelsR))
  np, nr, nnz = Ref{Int32}(0), Ref{Int32}(0), Ref{Int64}(0)
  check(ccall((:nd_bs_plan_sizes, LIB), Int32, (Ptr{Cvoid}, Ref{Int32}, Ref{Int32}, Ref{Int64}), plan[], np, nr, nnz))
  NR = length(labelsR)
  blocksR = Vector{Int32}(undef, max(1, nr[] * NR))
  offsR = Vector{Int64}(undef, max(1, nr[]))
  check(ccall((:nd_bs_plan_get, LIB), Int32, (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int64}, Ptr{Int32}), plan[], blocksR, offsR, C_NULL))
  indsR = NDTensors.contract_inds(inds(T1), labels1, inds(T2), labels2, labelsR)
  boffsR = BlockOffsets{NR}()
  for k in 1:nr[]
    insert!(boffsR, Block(ntuple(i -> UInt(blocksR[(k - 1) * NR + i]), NR)), offsR[k])
  end
  R = BlockSparseTensor(NDTensors.BlockSparse(GB300Vector(undef, nnz[]), boffsR), indsR)
  if np[] > 0
    check(ccall((:nd_bs_contract_f64, LIB), Int32, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Float64, Int32),
                handle(), plan[], data(R).ptr, data(T1).ptr, data(T2).ptr, 1.0, PRECISION[]))
  end
  ccall((:nd_bs_plan_destroy, LIB), Int32, (Ptr{Cvoid},), plan[])
  return R
end

const GB300BlockSparseMatrix = Tensor{Float64,2,<:NDTensors.BlockSparse{Float64,<:GB300Vector}}
isgb300(T::Tensor) = data(T) isa Union{GB300Vector,GB300View}
isgb300(x) = isgb300(NDTensors.tensor(x))        # an ITensor: its storage
const GB300BlockSparseTensor = BlockSparseTensor{Float64,N,<:NDTensors.BlockSparse{Float64,<:GB300Vector}} where {N}

# rows, columns and offsets of the nonzero blocks of a block-sparse matrix, in block order
function matrix_blocks(T)
  i1, i2 = ind(T, 1), ind(T, 2)
  nzb = collect(nzblocks(T))
  rows = Int64[blockdim(i1, b[1]) for b in nzb]
  cols = Int64[blockdim(i2, b[2]) for b in nzb]
  offs = Int64[NDTensors.offset(T, b) for b in nzb]
  return nzb, rows, cols, offs
end

# truncate! on the device (NDTensors/src/truncate.jl:15-20 copies GPU spectra to the
# CPU instead): the kept prefix of P is returned as a view of P.
function NDTensors.truncate!!(::Type{<:Union{GB300Vector,GB300View}}, P::AbstractVector;
                              mindim=nothing, maxdim=nothing, cutoff=nothing,
                              use_absolute_cutoff=nothing, use_relative_cutoff=nothing)
  n, terr, dcut = Ref{Int32}(0), Ref{Float64}(0), Ref{Float64}(0)
  check(ccall((:nd_truncate_f64, LIB), Int32,
              (Ptr{Cvoid}, Ptr{Float64}, Int32, Int32, Int32, Float64, Int32, Int32, Ref{Int32}, Ref{Float64}, Ref{Float64}),
              handle(), P.ptr, length(P), Int32(something(mindim, 1)), Int32(something(maxdim, -1)),
              Float64(something(cutoff, -1.0)), Int32(something(use_absolute_cutoff, false)),
              Int32(something(use_relative_cutoff, true)), n, terr, dcut))
  parent = P isa GB300View ? P.parent : P
  return GB300View(parent, P.ptr, Int(n[])), terr[], dcut[]
end

# Blockwise SVD with truncation (NDTensors/src/blocksparse/linearalgebra.jl:45-215): one
# batched device call computes every block's SVD, the pooled sort, truncate! and the kept
# dimensions; this method builds the reference's output structure from them.  Returns
# `nothing` when a block does not converge, as the reference does.
function LinearAlgebra.svd(T::GB300BlockSparseMatrix; min_blockdim=nothing, mindim=nothing, maxdim=nothing,
                           cutoff=nothing, alg=nothing, use_absolute_cutoff=nothing, use_relative_cutoff=nothing)
  nzb, rows, cols, offs = matrix_blocks(T)
  nb = length(nzb)
  ks = min.(rows, cols)
  U = GB300Vector(undef, sum(rows .* ks))
  S = GB300Vector(undef, sum(ks))
  V = GB300Vector(undef, sum(cols .* ks))
  kept = zeros(Int32, max(nb, 1))
  spec = Vector{Float64}(undef, max(sum(ks), 1))
  slen, terr, dcut = Ref{Int32}(0), Ref{Float64}(0), Ref{Float64}(0)
  st = ccall((:nd_bs_svd_f64, LIB), Int32,
             (Ptr{Cvoid}, Int32, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
              Ptr{Float64}, Int32, Int32, Float64, Int32, Int32, Int32, Ptr{Int32}, Ptr{Float64}, Ref{Int32},
              Ref{Float64}, Ref{Float64}),
             handle(), nb, rows, cols, offs, data(T).ptr, U.ptr, S.ptr, V.ptr,
             Int32(something(mindim, 1)), Int32(something(maxdim, -1)), Float64(something(cutoff, -1.0)),
             Int32(something(use_absolute_cutoff, false)), Int32(something(use_relative_cutoff, true)),
             Int32(something(min_blockdim, 0)), kept, spec, slen, terr, dcut)
  st == ND_ERR_NOCONV && return nothing
  check(st)
  # blocks whose kept dimension is 0 are dropped (linearalgebra.jl:86-114)
  surv = [n for n in 1:nb if kept[n] > 0]
  i1, i2 = ind(T, 1), ind(T, 2)
  uind = dag(sim(i1))
  vind = dag(sim(i2))
  resize!(uind, length(surv))
  resize!(vind, length(surv))
  for (n, m) in enumerate(surv)
    setblock!(uind, resize(block(i1, nzb[m][1]), Int(kept[m])), n)
    setblock!(vind, resize(block(i2, nzb[m][2]), Int(kept[m])), n)
  end
  nzblocksU = [Block(nzb[m][1], UInt(n)) for (n, m) in enumerate(surv)]
  nzblocksS = [Block(UInt(n), UInt(n)) for n in 1:length(surv)]
  nzblocksV = [Block(nzb[m][2], UInt(n)) for (n, m) in enumerate(surv)]
  indsU = NDTensors.setindex(inds(T), uind, 2)
  indsV = NDTensors.permute(NDTensors.setindex(inds(T), vind, 1), (2, 1))
  indsS = NDTensors.setindex(NDTensors.setindex(inds(T), dag(uind), 1), dag(vind), 2)
  # the library wrote the kept blocks in this order, each column-major m x k / n x k,
  # which is exactly the BlockOffsets layout of nzblocksU / nzblocksV
  bU, _ = NDTensors.blockoffsets(nzblocksU, indsU)
  bV, _ = NDTensors.blockoffsets(nzblocksV, indsV)
  bS = BlockOffsets{2}()
  o = 0
  for (n, m) in enumerate(surv)
    insert!(bS, nzblocksS[n], o)
    o += Int(kept[m])
  end
  Ut = BlockSparseTensor(NDTensors.BlockSparse(U, bU), indsU)
  St = DiagBlockSparseTensor(NDTensors.DiagBlockSparse(S, bS), indsS)
  Vt = BlockSparseTensor(NDTensors.BlockSparse(V, bV), indsV)
  return Ut, St, Vt, Spectrum(spec[1:slen[]], terr[])
end

# Blockwise QR through qx (NDTensors/src/blocksparse/linearalgebra.jl:351-415): one batched
# Householder launch; Q blocks (b1, n) of m x k, R blocks (n, b2) of k x n_cols.
function qx_gb300(T::GB300BlockSparseMatrix; positive=nothing)
  nzb, rows, cols, offs = matrix_blocks(T)
  nb = length(nzb)
  ks = min.(rows, cols)
  Q = GB300Vector(undef, sum(rows .* ks))
  X = GB300Vector(undef, sum(cols .* ks))
  check(ccall((:nd_bs_qr_f64, LIB), Int32,
              (Ptr{Cvoid}, Int32, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int32),
              handle(), nb, rows, cols, offs, data(T).ptr, Q.ptr, X.ptr, Int32(something(positive, false))))
  itl = ind(T, 1)
  iq = dag(sim(itl))
  resize!(iq, nb)
  for (n, b) in enumerate(nzb)
    setblock!(iq, resize(block(itl, b[1]), ks[n]), n)
  end
  indsQ = NDTensors.setindex(inds(T), iq, 2)
  indsX = NDTensors.setindex(inds(T), dag(iq), 1)
  nzblocksQ = [Block(b[1], UInt(n)) for (n, b) in enumerate(nzb)]
  nzblocksX = [Block(UInt(n), b[2]) for (n, b) in enumerate(nzb)]
  bQ, _ = NDTensors.blockoffsets(nzblocksQ, indsQ)
  bX, _ = NDTensors.blockoffsets(nzblocksX, indsX)
  return BlockSparseTensor(NDTensors.BlockSparse(Q, bQ), indsQ), BlockSparseTensor(NDTensors.BlockSparse(X, bX), indsX)
end
LinearAlgebra.qr(T::GB300BlockSparseMatrix; kwargs...) = qx_gb300(T; kwargs...)

# plan of one block-sparse contraction (kept by the pullback)
function bs_plan(T1, labels1, T2, labels2, labelsR)
  a1 = desc_arrays(T1)
  a2 = desc_arrays(T2)
  plan = Ref{Ptr{Cvoid}}(C_NULL)
  GC.@preserve a1 a2 begin
    d1 = Ref(BsDesc(length(a1[1]), pointer(a1[1]), pointer(a1[2]), a1[5], pointer(a1[3]), pointer(a1[4])))
    d2 = Ref(BsDesc(length(a2[1]), pointer(a2[1]), pointer(a2[2]), a2[5], pointer(a2[3]), pointer(a2[4])))
    check(ccall((:nd_bs_plan_create, LIB), Int32,
                (Ptr{Cvoid}, Ref{BsDesc}, Ptr{Int32}, Ref{BsDesc}, Ptr{Int32}, Int32, Ptr{Int32}, Ref{Ptr{Cvoid}}),
                handle(), d1, Int32[labels1...], d2, Int32[labels2...], length(labelsR), Int32[labelsR...], plan))
  end
  return plan[]
end

# Pullback of R = contract(T1, T2): both cotangents (R̄ * T2 over T2's free labels and
# T1 * R̄) in one grouped launch, with the structures of T1 and T2
# (ext/ITensorsChainRulesCoreExt/itensor.jl:94-103; real FP64, so dag is the identity).
function contract_pullback_gb300(T1, labels1, T2, labels2, labelsR, R̄)
  plan = bs_plan(T1, labels1, T2, labels2, labelsR)
  T̄1 = BlockSparseTensor(NDTensors.BlockSparse(GB300Vector(undef, length(data(T1))), blockoffsets(T1)), inds(T1))
  T̄2 = BlockSparseTensor(NDTensors.BlockSparse(GB300Vector(undef, length(data(T2))), blockoffsets(T2)), inds(T2))
  st = ccall((:nd_bs_contract_adjoint_f64, LIB), Int32,
             (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int32),
             handle(), plan, data(R̄).ptr, data(T1).ptr, data(T2).ptr, data(T̄1).ptr, data(T̄2).ptr, PRECISION[])
  ccall((:nd_bs_plan_destroy, LIB), Int32, (Ptr{Cvoid},), plan)
  check(st)
  return T̄1, T̄2
end

function ChainRulesCore.rrule(::typeof(NDTensors.contract), T1::GB300BlockSparseTensor, labels1,
                              T2::GB300BlockSparseTensor, labels2, labelsR=contract_labels(labels1, labels2))
  R = NDTensors.contract(T1, labels1, T2, labels2, labelsR)
  function contract_pullback(R̄)
    T̄1, T̄2 = contract_pullback_gb300(T1, labels1, T2, labels2, labelsR, ChainRulesCore.unthunk(R̄))
    return (NoTangent(), T̄1, NoTangent(), T̄2, NoTangent(), NoTangent())
  end
  return R, contract_pullback
end

# ---- BlockSparse x DiagBlockSparse (NDTensors/src/blocksparse/diagblocksparse.jl:601-696) ----
# D is passed as its diagonals; one launch writes R (no dense expansion of D, no GEMM).
const GB300DiagBlockSparseTensor = DiagBlockSparseTensor{Float64,N,<:NDTensors.DiagBlockSparse{Float64,<:GB300Vector}} where {N}

function NDTensors.contract(T1::GB300BlockSparseTensor, labels1, T2::GB300DiagBlockSparseTensor, labels2,
                            labelsR=contract_labels(labels1, labels2))
  plan = bs_plan(T1, labels1, T2, labels2, labelsR)
  np, nr, nnz = Ref{Int32}(0), Ref{Int32}(0), Ref{Int64}(0)
  check(ccall((:nd_bs_plan_sizes, LIB), Int32, (Ptr{Cvoid}, Ref{Int32}, Ref{Int32}, Ref{Int64}), plan, np, nr, nnz))
  NR = length(labelsR)
  blocksR = Vector{Int32}(undef, max(1, nr[] * NR))
  offsR = Vector{Int64}(undef, max(1, nr[]))
  check(ccall((:nd_bs_plan_get, LIB), Int32, (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int64}, Ptr{Int32}), plan, blocksR, offsR, C_NULL))
  indsR = NDTensors.contract_inds(inds(T1), labels1, inds(T2), labels2, labelsR)
  boffsR = BlockOffsets{NR}()
  for k in 1:nr[]
    insert!(boffsR, Block(ntuple(i -> UInt(blocksR[(k - 1) * NR + i]), NR)), offsR[k])
  end
  R = BlockSparseTensor(NDTensors.BlockSparse(GB300Vector(undef, nnz[]), boffsR), indsR)
  diag_offs = Int64[NDTensors.offset(T2, b) for b in nzblocks(T2)]
  st = np[] > 0 ? ccall((:nd_bs_contract_diag_f64, LIB), Int32,
                        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int64}, Float64),
                        handle(), plan, data(R).ptr, data(T1).ptr, data(T2).ptr, diag_offs, 1.0) : Int32(0)
  ccall((:nd_bs_plan_destroy, LIB), Int32, (Ptr{Cvoid},), plan)
  check(st)
  return R
end
NDTensors.contract(T1::GB300DiagBlockSparseTensor, labels1, T2::GB300BlockSparseTensor, labels2,
                   labelsR=contract_labels(labels1, labels2)) = NDTensors.contract(T2, labels2, T1, labels1, labelsR)

# ---- blockwise Hermitian eigen (NDTensors/src/blocksparse/linearalgebra.jl:221-348) ----
# One device call: every block's eigendecomposition, the pooled |lambda| sort,
# truncate! and the kept dimensions; this method builds the reference's output
# structure (D on (l, r), V on (dag(i2), r), blocks (n, n) and (b, n)).
function LinearAlgebra.eigen(X::Union{Hermitian{Float64,<:GB300BlockSparseMatrix},GB300BlockSparseMatrix};
                             min_blockdim=nothing, mindim=nothing, maxdim=nothing, cutoff=nothing,
                             use_absolute_cutoff=nothing, use_relative_cutoff=nothing)
  T = X isa Hermitian ? parent(X) : X
  nzb, rows, cols, offs = matrix_blocks(T)
  all(b -> b[1] == b[2], nzb) || error("Eigen currently only supports block diagonal matrices.")
  nb = length(nzb)
  D = GB300Vector(undef, sum(rows))
  V = GB300Vector(undef, sum(rows .* rows))
  kept = zeros(Int32, max(nb, 1))
  spec = Vector{Float64}(undef, max(sum(rows), 1))
  slen, terr, dcut = Ref{Int32}(0), Ref{Float64}(0), Ref{Float64}(0)
  check(ccall((:nd_bs_eigen_f64, LIB), Int32,
              (Ptr{Cvoid}, Int32, Ptr{Int64}, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int32, Int32,
               Float64, Int32, Int32, Int32, Ptr{Int32}, Ptr{Float64}, Ref{Int32}, Ref{Float64}, Ref{Float64}),
              handle(), nb, rows, offs, data(T).ptr, D.ptr, V.ptr,
              Int32(something(mindim, 1)), Int32(something(maxdim, -1)), Float64(something(cutoff, -1.0)),
              Int32(something(use_absolute_cutoff, false)), Int32(something(use_relative_cutoff, true)),
              Int32(something(min_blockdim, 0)), kept, spec, slen, terr, dcut))
  surv = [n for n in 1:nb if kept[n] > 0]
  i1, i2 = inds(T)
  l = sim(i1)
  deleteat!(l, setdiff(1:NDTensors.nblocks(l), Int[nzb[m][1] for m in surv]))
  for (n, m) in enumerate(surv)
    NDTensors.setblockdim!(l, Int(kept[m]), n)
  end
  r = dag(sim(l))
  indsD, indsV = (l, r), (dag(i2), r)
  nzblocksD = [Block(UInt(n), UInt(n)) for n in 1:length(surv)]
  nzblocksV = [Block(nzb[m][1], UInt(n)) for (n, m) in enumerate(surv)]
  # the library wrote the kept blocks in this order (V blocks column-major dims x kept)
  bV, _ = NDTensors.blockoffsets(nzblocksV, indsV)
  bD = BlockOffsets{2}()
  o = 0
  for (n, m) in enumerate(surv)
    insert!(bD, nzblocksD[n], o)
    o += Int(kept[m])
  end
  Dt = DiagBlockSparseTensor(NDTensors.DiagBlockSparse(D, bD), indsD)
  Vt = BlockSparseTensor(NDTensors.BlockSparse(V, bV), indsV)
  return Dt, Vt, Spectrum(spec[1:slen[]], terr[])
end

# ---- vector space (ext/ITensorsVectorInterfaceExt/ITensorsVectorInterfaceExt.jl:5-84) ----
# inner / norm / scale! / add! of ITensors reach the storage as LinearAlgebra.dot, norm,
# rmul! and axpby! on the data vector; each is one library launch (deterministic
# reduction order), the scalar results come back to the host.
const GB300Data = Union{GB300Vector,GB300View}

function LinearAlgebra.dot(x::GB300Data, y::GB300Data)
  length(x) == length(y) || throw(DimensionMismatch("dot: lengths $(length(x)) and $(length(y))"))
  out = GB300Vector(undef, 1)
  check(ccall((:nd_vec_inner_f64, LIB), Int32, (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
              handle(), length(x), x.ptr, y.ptr, out.ptr))
  return Array(out)[1]
end

function LinearAlgebra.norm(x::GB300Data)
  out = GB300Vector(undef, 1)
  check(ccall((:nd_vec_norm_f64, LIB), Int32, (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}),
              handle(), length(x), x.ptr, out.ptr))
  return Array(out)[1]
end

function LinearAlgebra.rmul!(x::GB300Data, a::Real)
  check(ccall((:nd_vec_scale_f64, LIB), Int32, (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Float64, Ptr{Float64}, Int32),
              handle(), length(x), x.ptr, x.ptr, Float64(a), C_NULL, Int32(0)))
  return x
end

function LinearAlgebra.axpby!(a::Real, x::GB300Data, b::Real, y::GB300Data)
  length(x) == length(y) || throw(DimensionMismatch("axpby!: lengths $(length(x)) and $(length(y))"))
  check(ccall((:nd_vec_add_f64, LIB), Int32, (Ptr{Cvoid}, Int64, Ptr{Float64}, Ptr{Float64}, Float64, Float64),
              handle(), length(x), x.ptr, y.ptr, Float64(a), Float64(b)))
  return y
end

LinearAlgebra.axpy!(a::Real, x::GB300Data, y::GB300Data) = LinearAlgebra.axpby!(a, x, 1.0, y)

end # module
