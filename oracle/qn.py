"""U(1) quantum-number index model (oracle restatement).

A QN index is an ordered list of sectors ``(charge, dim)`` plus an arrow
(``+1`` = Out, ``-1`` = In).  Block numbers are 1-based, as Julia's ``Block``.

Follows:
  src/qn/qnindex.jl:248        flux(i, b) = dir(i) * qn(i, b)
  src/indexset.jl:876-883      flux(inds, block) = sum of per-index fluxes
  NDTensors/src/blocksparse/blockdims.jl:104-106   eachblock = CartesianIndices (column-major)
  src/qn/qnindexset.jl:9-18    nzblocks(qn, inds): eachblock filtered by flux
  src/qn/qnindex.jl:359-379    outer / tensor product of QN spaces (first index fastest)
  src/qn/qnindex.jl:407-426    combineblocks: stable sortperm by QN, merge equal QNs
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass, field


@dataclass(frozen=True)
class QNIndex:
    sectors: tuple            # ((charge, dim), ...)
    arrow: int = 1            # +1 Out, -1 In
    tag: str = ""             # identity for labelling; equal tags == same index
    prime: int = 0

    @property
    def dims(self):
        return tuple(d for _, d in self.sectors)

    @property
    def nblocks(self):
        return len(self.sectors)

    @property
    def dim(self):
        return sum(self.dims)

    def dag(self):
        return QNIndex(self.sectors, -self.arrow, self.tag, self.prime)

    def primed(self, n=1):
        return QNIndex(self.sectors, self.arrow, self.tag, self.prime + n)

    def ident(self):
        """Identity used for index matching (arrow excluded, as ITensor's ==)."""
        return (self.tag, self.prime, self.sectors)

    def flux(self, b):
        """Flux of 1-based block b (src/qn/qnindex.jl:248)."""
        return self.arrow * self.sectors[b - 1][0]


def flux(inds, block):
    """Total flux of a block (src/indexset.jl:876-883)."""
    return sum(ix.flux(b) for ix, b in zip(inds, block))


def eachblock(inds):
    """All block tuples in column-major order (first index fastest), 1-based
    (NDTensors/src/blocksparse/blockdims.jl:104-106)."""
    ranges = [range(1, ix.nblocks + 1) for ix in inds]
    for t in itertools.product(*reversed(ranges)):
        yield tuple(reversed(t))


def nzblocks(qn, inds):
    """Blocks with the requested flux, in eachblock order (src/qn/qnindexset.jl:9-18)."""
    return [b for b in eachblock(inds) if flux(inds, b) == qn]


def blockdims(inds, block):
    """Per-dimension dims of a block (blockdims.jl:143-148)."""
    return tuple(ix.sectors[b - 1][1] for ix, b in zip(inds, block))


def tensor_product_sectors(i1, i2, arrow=None):
    """Space of the fused index i1 (x) i2 (src/qn/qnindex.jl:359-379).

    Each factor's charges are first multiplied by its own arrow, the product
    iterates the first factor fastest, then the result is multiplied by the new
    arrow (Out unless both factors share an arrow).
    """
    if arrow is None:
        arrow = i1.arrow if i1.arrow == i2.arrow else 1
    out = []
    for (q2, d2) in i2.sectors:
        for (q1, d1) in i1.sectors:
            out.append((arrow * (i1.arrow * q1 + i2.arrow * q2), d1 * d2))
    return tuple(out), arrow


def fuse(indices, arrow=None, tag="CMB"):
    """Uncombined fused index of several QN indices (left fold of the pairwise product)."""
    if arrow is None:
        a0 = indices[0].arrow
        arrow = a0 if all(ix.arrow == a0 for ix in indices) else 1
    cur = QNIndex(tuple((ix_q * indices[0].arrow * arrow, d) for ix_q, d in indices[0].sectors),
                  arrow, tag)
    for ix in indices[1:]:
        sec, _ = tensor_product_sectors(cur, ix, arrow)
        cur = QNIndex(sec, arrow, tag)
    return cur


def combineblocks(sectors):
    """(combined sectors, perm, comb) of src/qn/qnindex.jl:407-426.

    perm is a stable ascending sort of the sectors by charge (1-based); comb[i]
    is the combined block number of sorted position i (1-based).
    """
    perm = sorted(range(len(sectors)), key=lambda i: sectors[i][0])  # Python sort is stable
    sp = [sectors[i] for i in perm]
    combined = [list(sp[0])]
    comb = [1]
    for i in range(1, len(sp)):
        if sp[i][0] == sp[i - 1][0]:
            combined[-1][1] += sp[i][1]
        else:
            combined.append(list(sp[i]))
        comb.append(len(combined))
    return tuple((q, d) for q, d in combined), [p + 1 for p in perm], comb


@dataclass
class Space:
    """Block dims of a (possibly non-QN) block index: only dims matter to NDTensors."""
    dims: tuple
    charges: tuple = field(default=None)
