"""Reverse-mode rule for contraction (the ChainRulesCore rrule of ITensors).

Mirrors ext/ITensorsChainRulesCoreExt/itensor.jl:94-103:

    rrule(contract, x1, x2):  y = x1 * x2
        pullback(ybar) = (ybar * dag(x2), dag(x1) * ybar)

Both cotangents are contractions; the library runs them as ONE grouped launch
over the forward plan's block pairs (nd_bs_contract_adjoint_f64).  For real
FP64 data dag() leaves values unchanged.  Intermediate permutations are never
stored: each pullback recomputes them through its own addressing.

`contract_rrule` returns (y, pullback); `Contract` is the same rule as a
torch.autograd.Function over flat device data, so torch's autograd can chain it.
Dense tensors are handled as one-block block-sparse tensors.
"""
from __future__ import annotations

import ctypes as C

from ._lib import PRECISIONS
from .contract import contract_blocksparse, contract_labels, get_plan
from .tensors import BlockSparseTensor, DenseTensor


def as_blocksparse(T):
    if isinstance(T, BlockSparseTensor):
        return T
    if isinstance(T, DenseTensor):
        return BlockSparseTensor([(int(d),) for d in T.dims], [tuple(1 for _ in T.dims)], [0], T.data)
    raise TypeError("expected DenseTensor or BlockSparseTensor")


def _prec(p):
    return p if isinstance(p, int) else PRECISIONS[p]


def pullback_data(plan, T1, T2, ybar_data, precision="fp64"):
    """Cotangent data (flat) of T1 and T2 for the forward plan T1 * T2."""
    import torch
    a_bar = torch.empty_like(T1.data)
    b_bar = torch.empty_like(T2.data)
    plan.h.call("nd_bs_contract_adjoint_f64", plan.ptr, C.c_void_p(ybar_data.data_ptr()),
                C.c_void_p(T1.data.data_ptr()), C.c_void_p(T2.data.data_ptr()),
                C.c_void_p(a_bar.data_ptr()), C.c_void_p(b_bar.data_ptr()), _prec(precision))
    return a_bar, b_bar


def contract_rrule(T1, l1, T2, l2, lr=None, precision="fp64"):
    """(y, pullback) for y = contract(T1, l1, T2, l2, lr); pullback(ybar) -> (T1bar, T2bar)."""
    dense = isinstance(T1, DenseTensor)
    B1, B2 = as_blocksparse(T1), as_blocksparse(T2)
    l1, l2 = tuple(l1), tuple(l2)
    lr = contract_labels(l1, l2) if lr is None else tuple(lr)
    plan = get_plan(B1, l1, B2, l2, lr)
    y = contract_blocksparse(B1, l1, B2, l2, lr, precision=precision, plan=plan)

    def pullback(ybar):
        yb = ybar.data if hasattr(ybar, "data") and not hasattr(ybar, "data_ptr") else ybar
        a_bar, b_bar = pullback_data(plan, B1, B2, yb, precision)
        if dense:
            return DenseTensor(T1.dims, a_bar), DenseTensor(T2.dims, b_bar)
        return (BlockSparseTensor(B1.inds, B1.blocks, B1.offsets, a_bar),
                BlockSparseTensor(B2.inds, B2.blocks, B2.offsets, b_bar))

    if dense:
        y = DenseTensor(tuple(i[0] for i in y.inds), y.data)
    return y, pullback


def _torch_fn():
    import torch

    class Contract(torch.autograd.Function):
        """Differentiable contraction of flat device data with a fixed structure."""

        @staticmethod
        def forward(ctx, a, b, s1, l1, s2, l2, lr, precision):
            T1 = BlockSparseTensor(s1[0], s1[1], s1[2], a)
            T2 = BlockSparseTensor(s2[0], s2[1], s2[2], b)
            plan = get_plan(T1, l1, T2, l2, lr)
            y = contract_blocksparse(T1, l1, T2, l2, lr, precision=precision, plan=plan)
            ctx.save_for_backward(a, b)
            ctx.meta = (s1, l1, s2, l2, lr, precision, plan)
            return y.data

        @staticmethod
        def backward(ctx, ybar):
            a, b = ctx.saved_tensors
            s1, l1, s2, l2, lr, precision, plan = ctx.meta
            T1 = BlockSparseTensor(s1[0], s1[1], s1[2], a)
            T2 = BlockSparseTensor(s2[0], s2[1], s2[2], b)
            a_bar, b_bar = pullback_data(plan, T1, T2, ybar.contiguous(), precision)
            return a_bar, b_bar, None, None, None, None, None, None

    return Contract


_Contract = None


def contract_autograd(a, s1, l1, b, s2, l2, lr=None, precision="fp64"):
    """Flat-data differentiable contract: s1/s2 are (inds, blocks, offsets) structures.

    Returns the flat output data; the output structure is get_plan(...)'s."""
    global _Contract
    if _Contract is None:
        _Contract = _torch_fn()
    l1, l2 = tuple(l1), tuple(l2)
    lr = contract_labels(l1, l2) if lr is None else tuple(lr)
    return _Contract.apply(a, b, s1, l1, s2, l2, lr, precision)


def dense_structure(dims):
    """(inds, blocks, offsets) of a dense tensor seen as one block."""
    return ([(int(d),) for d in dims], [tuple(1 for _ in dims)], [0])
