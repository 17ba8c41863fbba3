"""``truncate!`` restated line by line (oracle).

Follows NDTensors/src/truncate.jl:23-107 (identical copy at
NDTensors/src/lib/RankFactorization/src/truncate_spectrum.jl:23-107) with the
defaults of NDTensors/src/default_kwargs.jl:6-11 (mindim = 1, maxdim =
length(P), cutoff = typemin, relative cutoff on, absolute cutoff off).

``P`` is a list of floats sorted descending (squared singular values).  Returns
(truncated list, truncerr, docut).  Summation ``sum(P)`` uses left-to-right
order; Julia's ``sum`` is pairwise with SIMD reassociation, so ``scale`` can
differ from the reference in the last bit (decisions differ only on exact ties).
"""
from __future__ import annotations

import math


def truncate(P, mindim=None, maxdim=None, cutoff=None, use_absolute_cutoff=None,
             use_relative_cutoff=None):
    P = [float(x) for x in P]
    mindim = 1 if mindim is None else int(mindim)
    maxdim = len(P) if maxdim is None else int(maxdim)
    cutoff = -math.inf if cutoff is None else float(cutoff)
    use_absolute_cutoff = False if use_absolute_cutoff is None else bool(use_absolute_cutoff)
    use_relative_cutoff = True if use_relative_cutoff is None else bool(use_relative_cutoff)

    origm = len(P)
    docut = 0.0
    if origm == 1:
        return P, 0.0, abs(P[0]) / 2

    s = math.copysign(1.0, P[0]) if P[0] != 0 else 0.0
    if s < 0:
        P = [x * s for x in P]

    for n in range(origm - 1, -1, -1):          # zero out negative weight from the end
        if P[n] >= 0.0:
            break
        P[n] = 0.0

    n = origm                                    # 1-based count kept
    truncerr = 0.0
    while n > maxdim:
        truncerr += P[n - 1]
        n -= 1

    if use_absolute_cutoff:
        while P[n - 1] <= cutoff and n > mindim:
            truncerr += P[n - 1]
            n -= 1
    else:
        scale = 1.0
        if use_relative_cutoff:
            scale = 0.0
            for x in P:
                scale += x
            if scale == 0.0:
                scale = 1.0
        while (truncerr + P[n - 1] <= cutoff * scale) and (n > mindim):
            truncerr += P[n - 1]
            n -= 1
        truncerr /= scale

    if n < 1:
        n = 1
    if n < origm:
        docut = (P[n - 1] + P[n]) / 2
        if abs(P[n - 1] - P[n]) < 1.0e-3 * P[n - 1]:
            docut += 1.0e-3 * P[n - 1]

    if s < 0:
        P = [x * s for x in P]
    return P[:n], truncerr, docut


def truncated_blockdim(svals, docut, singular_values=True, min_blockdim=None):
    """Kept size of one block (NDTensors/src/blocksparse/linearalgebra.jl:8-33)."""
    min_blockdim = 0 if min_blockdim is None else int(min_blockdim)
    full = len(svals)
    min_blockdim = min(min_blockdim, full)
    newdim = 0

    def v(k):
        return svals[k] ** 2 if singular_values else abs(svals[k])

    val = v(0) if full > 0 else -math.inf
    while newdim + 1 <= full and val > docut:
        newdim += 1
        if newdim + 1 <= full:
            val = v(newdim)
    if newdim < min_blockdim:
        newdim = min_blockdim
    return newdim
