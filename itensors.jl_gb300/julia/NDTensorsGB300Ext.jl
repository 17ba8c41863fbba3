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
#   svd(::BlockSparseMatrix) / qr(::BlockSparseMatrix)            (NDTensors/src/blocksparse/linearalgebra.jl:45-415)
#   rrule(contract, ::ITensor, ::ITensor)                         (ext/ITensorsChainRulesCoreExt/itensor.jl:94-103)
#
# Status: written against the C ABI in include/ndtensors_gb300.h; it has not been
# run (no Julia toolchain was available where this library was built and tested).
module NDTensorsGB300Ext

using NDTensors
using NDTensors: BlockSparseTensor, DenseTensor, Tensor, inds, data, blockoffsets, nzblocks,
    BlockOffsets, Block, blockdim, contract_labels
using NDTensors.Expose: Exposed, unexpose, expose
using LinearAlgebra

const LIB = get(ENV, "NDTENSORS_GB300_LIB", joinpath(@__DIR__, "..", "ndtensors_gb300", "libndtensors_gb300.so"))

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

function desc_arrays(T::BlockSparseTensor)
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
  a1 = desc_arrays(T1)
  a2 = desc_arrays(T2)
  GC.@preserve a1 a2 begin
    d1 = Ref(BsDesc(length(a1[1]), pointer(a1[1]), pointer(a1[2]), a1[5], pointer(a1[3]), pointer(a1[4])))
    d2 = Ref(BsDesc(length(a2[1]), pointer(a2[1]), pointer(a2[2]), a2[5], pointer(a2[3]), pointer(a2[4])))
    plan = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:nd_bs_plan_create, LIB), Int32,
                (Ptr{Cvoid}, Ref{BsDesc}, Ptr{Int32}, Ref{BsDesc}, Ptr{Int32}, Int32, Ptr{Int32}, Ref{Ptr{Cvoid}}),
                handle(), d1, Int32[labels1...], d2, Int32[labels2...], length(labelsR), Int32[labelsR...], plan))
  end
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

end # module
