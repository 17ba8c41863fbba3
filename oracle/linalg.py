"""Blockwise SVD / QR of a 2-index block-sparse matrix (oracle).

Follows:
  NDTensors/src/blocksparse/linearalgebra.jl:45-215   svd: per-block dense svd, pooled
      sorted s^2, truncate!!, per-block kept dims, dropped blocks, U (b1,n) S (n,n) V (b2,n)
  NDTensors/src/linearalgebra/linearalgebra.jl:80-160 dense svd (LAPACK gesdd by default)
  NDTensors/src/blocksparse/linearalgebra.jl:351-415  qx: per-block qr, new index dims = size(Q,2)
  NDTensors/src/linearalgebra/linearalgebra.jl:321-381 qr / qr_positive (sign fix of R's diagonal)
Dense factorizations use numpy.linalg (LAPACK gesdd / geqrf+orgqr), the same
LAPACK family as the reference's Julia stdlib.
"""
from __future__ import annotations

import numpy as np

from .truncate import truncate, truncated_blockdim


def svd_blocks(mats, mindim=None, maxdim=None, cutoff=None, use_absolute_cutoff=None,
               use_relative_cutoff=None, min_blockdim=None):
    """mats: list of dense 2-D blocks in nz-block order.

    Returns dict with U, S, V lists (truncated, dropped blocks removed), kept
    (per input block, 0 = dropped), spectrum (sorted s^2 after truncation),
    truncerr, docut.
    """
    Us, Ss, Vs = [], [], []
    d = []
    for m in mats:
        u, s, vt = np.linalg.svd(m, full_matrices=False)
        Us.append(u)
        Ss.append(s)
        Vs.append(vt.T)
        d.extend(s.tolist())
    d = sorted((x * x for x in d), reverse=True)
    kept = [len(s) for s in Ss]
    truncerr, docut = 0.0, 0.0
    if maxdim is not None or cutoff is not None:
        d, truncerr, docut = truncate(d, mindim=mindim, maxdim=maxdim, cutoff=cutoff,
                                      use_absolute_cutoff=use_absolute_cutoff,
                                      use_relative_cutoff=use_relative_cutoff)
        for n, s in enumerate(Ss):
            kept[n] = truncated_blockdim(s, docut, singular_values=True,
                                         min_blockdim=min_blockdim)
    out_u, out_s, out_v = [], [], []
    for n in range(len(mats)):
        k = kept[n]
        if k == 0:
            continue
        out_u.append(Us[n][:, :k])
        out_s.append(Ss[n][:k])
        out_v.append(Vs[n][:, :k])
    return dict(U=out_u, S=out_s, V=out_v, kept=kept, spectrum=d, truncerr=truncerr,
                docut=docut)


def eigen_blocks(mats, mindim=None, maxdim=None, cutoff=None, use_absolute_cutoff=None,
                 use_relative_cutoff=None, min_blockdim=None):
    """Blockwise Hermitian eigendecomposition (NDTensors/src/blocksparse/linearalgebra.jl:221-348).

    Per block a dense Hermitian eigen with eigenpairs sorted by |lambda| descending
    (NDTensors/src/linearalgebra/linearalgebra.jl:162-213), all |lambda| pooled and
    sorted descending, truncate!!, per block the leading eigenpairs with |lambda| > docut
    (_truncated_blockdim with singular_values = false, :8-33).  Returns dict with D
    (kept eigenvalues per surviving block), V, kept, spectrum (pooled |lambda| after
    truncation), truncerr, docut.
    """
    Ds, Vs, d = [], [], []
    for m in mats:
        lam, vec = np.linalg.eigh(m)
        order = np.argsort(-np.abs(lam), kind="stable")
        Ds.append(lam[order])
        Vs.append(vec[:, order])
        d.extend(np.abs(lam).tolist())
    d = sorted(d, reverse=True)
    kept = [len(x) for x in Ds]
    truncerr, docut = 0.0, 0.0
    if maxdim is not None or cutoff is not None:
        d, truncerr, docut = truncate(d, mindim=mindim, maxdim=maxdim, cutoff=cutoff,
                                      use_absolute_cutoff=use_absolute_cutoff,
                                      use_relative_cutoff=use_relative_cutoff)
        for n, lam in enumerate(Ds):
            kept[n] = truncated_blockdim(lam, docut, singular_values=False, min_blockdim=min_blockdim)
    out_d, out_v = [], []
    for n in range(len(mats)):
        k = kept[n]
        if k == 0:
            continue
        out_d.append(Ds[n][:k])
        out_v.append(Vs[n][:, :k])
    return dict(D=out_d, V=out_v, kept=kept, spectrum=d, truncerr=truncerr, docut=docut)


def qr_positive(m):
    """QR with non-negative diag(R) (linearalgebra.jl:374-381)."""
    q, r = np.linalg.qr(m, mode="reduced")
    dg = np.diag(r)
    signs = np.where(dg == 0, 1.0, np.sign(dg))
    return q * signs[None, :], signs[:, None] * r


def qr_blocks(mats, positive=False):
    out_q, out_r = [], []
    for m in mats:
        if positive:
            q, r = qr_positive(m)
        else:
            q, r = np.linalg.qr(m, mode="reduced")
        out_q.append(q)
        out_r.append(r)
    return out_q, out_r
