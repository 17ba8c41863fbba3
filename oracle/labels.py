"""ncon-style label logic of the contraction path (oracle restatement).

Follows:
  src/indexset.jl:672-707                           compute_contraction_labels
  NDTensors/src/tensoroperations/contraction_logic.jl:5-34   contract_labels
  NDTensors/src/tensoroperations/contraction_logic.jl:36-55  _contract_inds!
  NDTensors/src/blocksparse/contract_utilities.jl:28-55      find_matching_positions
"""
from __future__ import annotations


def compute_contraction_labels(inds_a, inds_b):
    """Labels for A and B given index identities (any hashable ids).

    Common indices get -1, -2, ... in the order they are found scanning A then B
    (src/indexset.jl:680-691); the remaining A indices, then B indices, get
    ncont+1, ncont+2, ... (src/indexset.jl:693-703).
    """
    la = [0] * len(inds_a)
    lb = [0] * len(inds_b)
    ncont = 0
    for i, ia in enumerate(inds_a):
        for j, ib in enumerate(inds_b):
            if ia == ib:
                ncont += 1
                la[i] = lb[j] = -ncont
    u = ncont
    for i in range(len(la)):
        if la[i] == 0:
            u += 1
            la[i] = u
    for j in range(len(lb)):
        if lb[j] == 0:
            u += 1
            lb[j] = u
    return tuple(la), tuple(lb)


def contract_labels(la, lb):
    """Output labels: positive labels of A in order, then of B (contraction_logic.jl:16-34)."""
    return tuple([l for l in la if l > 0] + [l for l in lb if l > 0])


def contract_inds(inds_a, la, inds_b, lb, lr):
    """Output index list picked by label, A searched first (contraction_logic.jl:36-55)."""
    out = []
    for l in lr:
        if l in la:
            out.append(inds_a[la.index(l)])
        else:
            out.append(inds_b[lb.index(l)])
    return out


def find_matching_positions(t1, t2):
    """1-based positions in t2 of each element of t1, 0 when absent; last match wins
    (contract_utilities.jl:45-55)."""
    res = [0] * len(t1)
    for p1, x in enumerate(t1):
        for p2, y in enumerate(t2):
            if x == y:
                res[p1] = p2 + 1
    return tuple(res)


def check_labels(la, lb, lr):
    """Argument validation the reference performs implicitly through its tuple types."""
    if len(set(la)) != len(la) or len(set(lb)) != len(lb):
        raise ValueError("repeated label within one tensor")
    if len(set(lr)) != len(lr):
        raise ValueError("repeated output label")
    free = [l for l in la if l not in lb] + [l for l in lb if l not in la]
    if sorted(free) != sorted(lr):
        raise ValueError("output labels must be exactly the uncontracted labels")
