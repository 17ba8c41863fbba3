"""NDTensors' contraction interface on the GB300 library.

Mirrors, name for name:
  contract(T1, labelsT1, T2, labelsT2[, labelsR])      NDTensors/src/tensoroperations/generic_tensor_operations.jl:87-118
  contract!(R, labelsR, T1, labelsT1, T2, labelsT2, a, b)  NDTensors/src/dense/tensoralgebra/contract.jl:160-216
  contract_labels(labelsT1, labelsT2)                  NDTensors/src/tensoroperations/contraction_logic.jl:5-34
  permutedims(T, perm), permutedims!(R, T, perm)       NDTensors/src/dense/densetensor.jl:212-275
  contract / contraction_output for BlockSparse        NDTensors/src/blocksparse/contract.jl:3-55
Python cannot use "!" in names: ``contract_`` is ``contract!``.
``precision`` is "fp64" (drop-in), "ozaki" or "bf16x3".
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as _libmod
from ._lib import MAX_RANK, PRECISIONS, BsDesc, handle, i32arr, i64arr
from .tensors import BlockSparseTensor, DenseTensor, blockoffsets


def contract_labels(l1, l2):
    """Positive labels of T1 then of T2 (contraction_logic.jl:16-34)."""
    return tuple([l for l in l1 if l > 0] + [l for l in l2 if l > 0])


def _prec(p):
    if isinstance(p, int):
        return p
    try:
        return PRECISIONS[p]
    except KeyError:
        raise ValueError(f"unknown precision {p!r}; expected one of {sorted(PRECISIONS)}")


def _out_dims(d1, l1, d2, l2, lr):
    out = []
    for l in lr:
        if l in l1:
            out.append(d1[l1.index(l)])
        elif l in l2:
            out.append(d2[l2.index(l)])
        else:
            raise ValueError(f"output label {l} appears in neither input")
    return tuple(out)


# ---------------------------------------------------------------------------
# dense
# ---------------------------------------------------------------------------

def permutedims_(R: DenseTensor, T: DenseTensor, perm, alpha=1.0, beta=0.0):
    """permutedims!(R, T, perm) with R = beta*R + alpha*permutedims(T, perm); perm is 1-based."""
    perm = tuple(int(p) for p in perm)
    if tuple(T.dims[p - 1] for p in perm) != tuple(R.dims):
        raise ValueError("permutedims!: R dims do not match permuted T dims")
    h = handle(T.data.device.index or 0)
    h.call("nd_permutedims_f64", C.c_void_p(R.ptr()), C.c_void_p(T.ptr()), len(T.dims), i64arr(T.dims),
           i32arr(perm), float(alpha), float(beta))
    return R


def permutedims(T: DenseTensor, perm):
    perm = tuple(int(p) for p in perm)
    R = DenseTensor.empty(tuple(T.dims[p - 1] for p in perm), T.data.device.index or 0)
    return permutedims_(R, T, perm)


def contract_(R: DenseTensor, labelsR, T1: DenseTensor, labels1, T2: DenseTensor, labels2,
              alpha=1.0, beta=0.0, precision="fp64"):
    """contract!(R, labelsR, T1, labelsT1, T2, labelsT2, alpha, beta) for Dense storage."""
    lr, l1, l2 = tuple(labelsR), tuple(labels1), tuple(labels2)
    if len(lr) != len(R.dims) or len(l1) != len(T1.dims) or len(l2) != len(T2.dims):
        raise ValueError("contract!: number of labels does not match the tensor ranks")
    h = handle(T1.data.device.index or 0)
    h.call("nd_contract_dense_f64",
           C.c_void_p(R.ptr()), len(R.dims), i64arr(R.dims), i32arr(lr),
           C.c_void_p(T1.ptr()), len(T1.dims), i64arr(T1.dims), i32arr(l1),
           C.c_void_p(T2.ptr()), len(T2.dims), i64arr(T2.dims), i32arr(l2),
           float(alpha), float(beta), _prec(precision))
    return R


# ---------------------------------------------------------------------------
# block sparse
# ---------------------------------------------------------------------------

class ContractionPlan:
    """Device-built block plan (contract_blockoffsets, contract_sequential.jl:1-41)."""

    def __init__(self, T1: BlockSparseTensor, l1, T2: BlockSparseTensor, l2, lr):
        self.l1, self.l2, self.lr = tuple(l1), tuple(l2), tuple(lr)
        self._custom_offsets = None
        if len(self.l1) != T1.rank or len(self.l2) != T2.rank:
            raise ValueError("contract: number of labels does not match the tensor ranks")
        self.h = handle(T1.data.device.index or 0)
        d1, d2 = T1.desc(), T2.desc()
        self.ptr = C.c_void_p()
        self.h.call("nd_bs_plan_create", C.byref(d1), i32arr(self.l1), C.byref(d2), i32arr(self.l2),
                    len(self.lr), i32arr(self.lr), C.byref(self.ptr))
        npairs, nR, nnzR = C.c_int32(), C.c_int32(), C.c_int64()
        self.h._check(self.h.lib.nd_bs_plan_sizes(self.ptr, C.byref(npairs), C.byref(nR), C.byref(nnzR)))
        self.npairs, self.nblocksR, self.nnzR = npairs.value, nR.value, nnzR.value
        rank = len(self.lr)
        br = np.empty(max(1, self.nblocksR * rank), dtype=np.int32)
        of = np.empty(max(1, self.nblocksR), dtype=np.int64)
        self._pairs_raw = np.empty(max(1, 3 * self.npairs), dtype=np.int32)
        P32, P64 = C.POINTER(C.c_int32), C.POINTER(C.c_int64)
        self.h._check(self.h.lib.nd_bs_plan_get(self.ptr, br.ctypes.data_as(P32), of.ctypes.data_as(P64),
                                                self._pairs_raw.ctypes.data_as(P32)))
        self._br = br[:self.nblocksR * rank].copy()         # kept as arrays: the output's descriptor
        self._of = of[:self.nblocksR].copy()
        self.blocksR = list(map(tuple, self._br.reshape(self.nblocksR, rank).tolist()))
        self.offsetsR = self._of.tolist()
        self._pairs = None
        self.indsR = [tuple(T1.inds[self.l1.index(l)]) if l in self.l1 else tuple(T2.inds[self.l2.index(l)])
                      for l in self.lr]
        from ._lib import _live_plans
        _live_plans.add(self)

    def output(self, data):
        """The output tensor on `data` (a flat device vector of nnzR), with its C-ABI
        descriptor built from the plan's arrays."""
        R = BlockSparseTensor(list(self.indsR), list(self.blocksR), list(self.offsetsR), data)
        if self._custom_offsets is None:
            R.set_desc_arrays(self._br, self._of)
        return R

    def pair_shapes(self, T1, T2):
        """(M, N, K, output block) of every block pair, in plan order."""
        out = []
        for (i1, i2, ir) in self.pairs:
            d1 = T1.blockdims(T1.blocks[i1])
            d2 = T2.blockdims(T2.blocks[i2])
            m = 1
            k = 1
            for d, l in zip(d1, self.l1):
                if l in self.l2:
                    k *= d
                else:
                    m *= d
            n = 1
            for d, l in zip(d2, self.l2):
                if l not in self.l1:
                    n *= d
            out.append((m, n, k, ir))
        return out

    @property
    def pairs(self):
        """(A block, B block, output block) of every contracted pair, in plan order."""
        if self._pairs is None:
            self._pairs = list(map(tuple, self._pairs_raw[:3 * self.npairs].reshape(self.npairs, 3).tolist()))
        return self._pairs

    def set_output_offsets(self, offsets):
        """Write the output blocks at these offsets (a caller's layout, e.g. psi's block
        order) instead of the first-appearance offsets."""
        offs = [int(o) for o in offsets]
        if len(offs) != self.nblocksR:
            raise ValueError("set_output_offsets: one offset per output block")
        self.h._check(self.h.lib.nd_bs_plan_set_output_offsets(self.ptr, i64arr(offs)))
        self.offsetsR = offs
        self._custom_offsets = offs

    def flops(self, T1, T2):
        return sum(2 * m * n * k for (m, n, k, _) in self.pair_shapes(T1, T2))

    def destroy(self):
        if self.ptr and self.h.ptr:
            self.h.lib.nd_bs_plan_destroy(self.ptr)
        self.ptr = C.c_void_p()

    def __del__(self):
        try:
            if _libmod._shutting_down:
                return
            self.destroy()
        except Exception:
            pass


_plan_cache = {}


def get_plan(T1, l1, T2, l2, lr):
    key = (T1.structure_key(), tuple(l1), T2.structure_key(), tuple(l2), tuple(lr))
    p = _plan_cache.get(key)
    if p is None:
        p = ContractionPlan(T1, l1, T2, l2, lr)
        if len(_plan_cache) > 256:
            _plan_cache.clear()
        _plan_cache[key] = p
    return p


def contract_blocksparse(T1, l1, T2, l2, lr=None, alpha=1.0, precision="fp64", plan=None, out=None):
    l1, l2 = tuple(l1), tuple(l2)
    lr = contract_labels(l1, l2) if lr is None else tuple(lr)
    plan = plan or get_plan(T1, l1, T2, l2, lr)
    R = out
    if R is None:
        import torch
        data = torch.empty(max(plan.nnzR, 1), dtype=torch.float64, device=T1.data.device)[:plan.nnzR]
        R = plan.output(data)
    if plan.npairs:
        handle(T1.data.device.index or 0)          # bind the handle to torch's current stream
        plan.h.call("nd_bs_contract_f64", plan.ptr, C.c_void_p(R.data.data_ptr()), C.c_void_p(T1.data.data_ptr()),
                    C.c_void_p(T2.data.data_ptr()), float(alpha), _prec(precision))
    return R


def contract_diag(T1: BlockSparseTensor, l1, D, l2, lr=None, alpha=1.0):
    """contract(::BlockSparseTensor, ::DiagBlockSparseTensor) (blocksparse/diagblocksparse.jl:601-696):
    the block plan and output structure of contraction_output, then one library kernel
    that scales / sums T1's entries by D's diagonal (no dense expansion of D)."""
    import torch
    l1, l2 = tuple(l1), tuple(l2)
    lr = contract_labels(l1, l2) if lr is None else tuple(lr)
    offs, _ = blockoffsets(D.blocks, D.inds)
    Ds = BlockSparseTensor(list(D.inds), list(D.blocks), offs, D.data)     # D's block structure for the planner
    plan = get_plan(T1, l1, Ds, l2, lr)
    data = torch.empty(max(plan.nnzR, 1), dtype=torch.float64, device=T1.data.device)[:plan.nnzR]
    R = BlockSparseTensor(list(plan.indsR), list(plan.blocksR), list(plan.offsetsR), data)
    if plan.nnzR:
        if not plan.npairs:
            handle(T1.data.device.index or 0).call("nd_memset0", C.c_void_p(data.data_ptr()), 8 * plan.nnzR)
        else:
            handle(T1.data.device.index or 0)
            plan.h.call("nd_bs_contract_diag_f64", plan.ptr, C.c_void_p(data.data_ptr()), C.c_void_p(T1.data.data_ptr()),
                        C.c_void_p(D.data.data_ptr()), i64arr(D.offsets), float(alpha))
    return R


def contract(T1, labels1, T2, labels2, labelsR=None, precision="fp64"):
    """contract(T1, labelsT1, T2, labelsT2[, labelsR]) for Dense, BlockSparse or
    BlockSparse x DiagBlockSparse storage, or a tensor with a CombinerTensor
    (linalg.contract_combiner; NDTensors/src/blocksparse/combiner.jl:25-143,
    NDTensors/src/combiner/contract.jl:14-77).

    A block-diagonal DiagBlockSparse operand runs on the library's diagonal kernel
    (contract_diag; NDTensors/src/blocksparse/diagblocksparse.jl:601-696) with the block
    plan and output structure of contraction_output; the result is exact (no
    precision choice applies: each output element is one product or a short sum)."""
    from .linalg import CombinerTensor, contract_combiner
    from .tensors import DiagBlockSparseTensor
    l1, l2 = tuple(labels1), tuple(labels2)
    first = isinstance(T1, CombinerTensor)
    if first:
        T1, l1, T2, l2 = T2, l2, T1, l1
    if isinstance(T2, CombinerTensor):
        if not isinstance(T1, (BlockSparseTensor, DenseTensor)):
            raise TypeError("contract: a combiner needs a Dense or BlockSparse partner")
        return contract_combiner(T1, l1, T2, l2, labelsR, combiner_first=first)[0]
    if isinstance(T1, DiagBlockSparseTensor):
        return contract(T2, l2, T1, l1, contract_labels(l2, l1) if labelsR is None else labelsR, precision)
    if isinstance(T2, DiagBlockSparseTensor):
        if not isinstance(T1, BlockSparseTensor):
            raise TypeError("contract: a DiagBlockSparse operand needs a BlockSparse partner")
        return contract_diag(T1, l1, T2, l2, labelsR)
    lr = contract_labels(l1, l2) if labelsR is None else tuple(labelsR)
    if isinstance(T1, BlockSparseTensor) and isinstance(T2, BlockSparseTensor):
        return contract_blocksparse(T1, l1, T2, l2, lr, precision=precision)
    if isinstance(T1, DenseTensor) and isinstance(T2, DenseTensor):
        R = DenseTensor.empty(_out_dims(T1.dims, l1, T2.dims, l2, lr), T1.data.device.index or 0)
        return contract_(R, lr, T1, l1, T2, l2, 1.0, 0.0, precision)
    raise TypeError("contract: both tensors must be Dense or both BlockSparse")


def permutedims_blocksparse(T: BlockSparseTensor, perm):
    """Block-sparse permutedims (blocksparsetensor.jl:465-470, blockoffsets.jl:103-111)."""
    import torch
    p0 = [int(p) - 1 for p in perm]
    inds = [T.inds[k] for k in p0]
    blocks = [tuple(b[k] for k in p0) for b in T.blocks]
    offs, nnz = blockoffsets(blocks, inds)
    R = BlockSparseTensor(inds, blocks, offs, torch.empty(max(nnz, 1), dtype=torch.float64,
                                                          device=T.data.device)[:nnz])
    h = handle(T.data.device.index or 0)
    d = T.desc()
    h.call("nd_bs_permutedims_f64", C.byref(d), C.c_void_p(T.data.data_ptr()), i32arr([int(p) for p in perm]),
           i64arr(offs), C.c_void_p(R.data.data_ptr()))
    return R
