"""Dense contraction and permutation (oracle restatement).

Arrays are numpy arrays indexed in the tensor's logical index order; storage
order does not matter to the values.  The reference's dense path is
``contract!`` -> ``_contract!`` = optional permutes + one BLAS ``gemm!``; the
permutation choices (ContractionProperties) change only rounding, so the oracle
computes the same sum with ``numpy.tensordot`` (OpenBLAS dgemm).

Follows:
  NDTensors/src/dense/tensoralgebra/contract.jl:160-216   contract! (scalar / outer / gemm branches)
  NDTensors/src/abstractarray/tensoralgebra/contract.jl:88-113   _contract_scalar_perm! (alpha/beta rules)
  NDTensors/src/abstractarray/tensoralgebra/contract.jl:115-188  _contract!
  NDTensors/src/array/permutedims.jl:5-24                 permutedims! with fused f(r, t)
"""
from __future__ import annotations

import numpy as np

from .labels import check_labels, contract_labels


def permutedims(t, perm1):
    """permutedims with a 1-based perm (Julia convention)."""
    return np.transpose(t, [p - 1 for p in perm1])


def permutedims_into(r, t, perm1, alpha=1.0, beta=0.0):
    """R = beta*R + alpha*permutedims(T, perm) with the reference's zero/one rules.

    beta == 0 overwrites R (NaN in R does not propagate), alpha == 0 leaves only
    the beta term (abstractarray/tensoralgebra/contract.jl:88-113).
    """
    p = permutedims(t, perm1)
    if beta == 0:
        if alpha == 0:
            r[...] = 0.0
        else:
            r[...] = alpha * p
    elif beta == 1:
        if alpha != 0:
            r[...] = r + alpha * p
    else:
        if alpha == 0:
            r[...] = beta * r
        else:
            r[...] = alpha * p + beta * r
    return r


def contract(a, la, b, lb, lr=None, alpha=1.0, beta=0.0, r=None):
    """R = alpha * contract(A, B) + beta * R with ncon labels.

    Negative labels are contracted; the output order is ``lr`` (default: the
    positive labels of A then B, contraction_logic.jl:16-34).
    """
    la, lb = tuple(la), tuple(lb)
    if lr is None:
        lr = contract_labels(la, lb)
    lr = tuple(lr)
    check_labels(la, lb, lr)
    cont = [l for l in la if l in lb]
    ax_a = [la.index(l) for l in cont]
    ax_b = [lb.index(l) for l in cont]
    prod = np.tensordot(a, b, axes=(ax_a, ax_b)) if cont else np.multiply.outer(a, b)
    lprod = [l for l in la if l not in cont] + [l for l in lb if l not in cont]
    prod = np.transpose(prod, [lprod.index(l) for l in lr]) if lr else prod
    if r is None:
        r = np.empty(prod.shape, dtype=np.float64)
        beta = 0.0
    if beta == 0:
        r[...] = alpha * prod if alpha != 1 else prod
    elif alpha == 0:
        r[...] = beta * r
    else:
        r[...] = alpha * prod + beta * r
    return r


def rel_frobenius_error(x, ref):
    ref = np.asarray(ref)
    den = np.linalg.norm(ref.ravel())
    num = np.linalg.norm((np.asarray(x) - ref).ravel())
    return float(num / den) if den > 0 else float(num)


def _drop_singletons(labels, dims):
    keep = [(l, d) for l, d in zip(labels, dims) if d != 1]
    return [l for l, _ in keep], [d for _, d in keep]


def contract_into(r, lr, a, la, b, lb, alpha=1.0, beta=0.0):
    """In-place ``contract!(R, labelsR, T1, labelsT1, T2, labelsT2, alpha, beta)``.

    Mirrors the branch order of NDTensors/src/dense/tensoralgebra/contract.jl:160-216:
    a one-element operand takes the scalar path (:100-150, singletons dropped before
    the permutation is derived), otherwise the general path.
    """
    if a.size == 1 or b.size == 1:
        if a.size == 1 and b.size == 1 and r.size == 1:
            s = float(a.reshape(-1)[0]) * float(b.reshape(-1)[0])
            rv = r.reshape(-1)
            if beta == 0:
                rv[0] = alpha * s
            elif alpha == 0:
                rv[0] = beta * rv[0]
            else:
                rv[0] = alpha * s + beta * rv[0]
            return r
        if a.size == 1:
            scal, t, lt = float(a.reshape(-1)[0]), b, lb
        else:
            scal, t, lt = float(b.reshape(-1)[0]), a, la
        lrr, drr = _drop_singletons(lr, r.shape)
        ltr, dtr = _drop_singletons(lt, t.shape)
        perm1 = [ltr.index(l) + 1 for l in lrr]
        rv = r.reshape(drr)            # dropping size-1 axes is always a view
        permutedims_into(rv, t.reshape(dtr), perm1, alpha * scal, beta)
        return r
    return contract(a, la, b, lb, lr, alpha=alpha, beta=beta, r=r)
