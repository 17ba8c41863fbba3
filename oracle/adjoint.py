"""Pullback of a pairwise contraction (oracle).

Follows ext/ITensorsChainRulesCoreExt/itensor.jl:94-103: for y = x1 * x2 the
cotangents are x1_bar = y_bar * dag(x2) and x2_bar = dag(x1) * y_bar, each a
contraction over the labels the two factors share.  For real FP64 data ``dag``
leaves values unchanged.  Labels here are arbitrary ids: shared ids contract.
"""
from __future__ import annotations

from .dense import contract


def contract_pullback(x1, l1, x2, l2, lr, ybar):
    l1, l2, lr = tuple(l1), tuple(l2), tuple(lr)
    x1bar = contract(ybar, lr, x2, l2, l1)
    x2bar = contract(x1, l1, ybar, lr, l2)
    return x1bar, x2bar
