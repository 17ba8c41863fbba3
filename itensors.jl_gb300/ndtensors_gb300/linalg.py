"""Blockwise factorizations and the block-sparse combiner on the GB300 library.

Mirrors:
  svd(T::BlockSparseMatrix; mindim, maxdim, cutoff, use_absolute_cutoff,
      use_relative_cutoff, min_blockdim)        NDTensors/src/blocksparse/linearalgebra.jl:45-215
  qr(T::BlockSparseMatrix; positive)            NDTensors/src/blocksparse/linearalgebra.jl:351-415
  truncate!(P; ...)                             NDTensors/src/truncate.jl:23-107
  combiner matricization (permutedims_combine)  NDTensors/src/blocksparse/blocksparsetensor.jl:537-638,
                                                src/qn/qnindex.jl:359-426
  uncombine                                     NDTensors/src/blocksparse/blocksparsetensor.jl:664-791
  contract(::BlockSparseTensor, ::CombinerTensor) NDTensors/src/blocksparse/combiner.jl:25-143
The factorizations, the spectrum sort and truncate! run on the device; only
the block structure (which blocks survive, their new dims) is host logic.
"""
from __future__ import annotations

import ctypes as C
import itertools

import numpy as np

from ._lib import ND_ERR_NOCONV, BlockCopy, MAX_RANK, NoConvergence, handle, i32arr, i64arr
from .tensors import BlockSparseTensor, blockoffsets


def _opt(x, none=-1):
    return none if x is None else x


class Spectrum:
    """Spectrum(eigs, truncerr) (NDTensors/src/lib/RankFactorization/src/spectrum.jl): the
    kept density-matrix eigenvalues of a decomposition (or None) and its truncation error."""

    def __init__(self, eigs, truncerr):
        self.eigs = None if eigs is None else np.asarray(eigs)
        self.truncerr = float(truncerr)


def eigs(spec: Spectrum):
    """eigs(::Spectrum)."""
    return spec.eigs


def truncerror(spec: Spectrum):
    """truncerror(::Spectrum)."""
    return spec.truncerr


def entropy(spec: Spectrum):
    """entropy(::Spectrum): -sum p log p over the eigenvalues above 1e-13; an error when
    the spectrum holds no eigenvalues (spectrum.jl:14-23)."""
    if spec.eigs is None:
        raise RuntimeError("Spectrum does not contain any eigenvalues, cannot compute the entropy")
    S = 0.0
    for p in spec.eigs:
        p = float(p)
        if p > 1.0e-13:
            S -= p * np.log(p)
    return S


def _matrix_blocks(T: BlockSparseTensor):
    if T.rank != 2:
        raise ValueError("factorizations need an order-2 block-sparse tensor")
    rows = [T.inds[0][b[0] - 1] for b in T.blocks]
    cols = [T.inds[1][b[1] - 1] for b in T.blocks]
    return rows, cols


def svd(T: BlockSparseTensor, mindim=None, maxdim=None, cutoff=None, use_absolute_cutoff=None,
        use_relative_cutoff=None, min_blockdim=None):
    """Returns (U, S, V, Spectrum, kept), or None when a block's SVD did not converge within
    the sweep limit (ND_ERR_NOCONV), as the reference's svd returns `nothing`
    (NDTensors/src/linearalgebra/linearalgebra.jl:120-127, blocksparse/linearalgebra.jl:65-67).

    U has inds (T.inds[0], u), S is a list of per-block singular values (Diag),
    V has inds (T.inds[1], v); u and v carry one block per surviving nz block.
    """
    import torch
    rows, cols = _matrix_blocks(T)
    nb = len(T.blocks)
    h = handle(T.data.device.index or 0)
    ks = [min(r, c) for r, c in zip(rows, cols)]
    dev = T.data.device
    U = torch.empty(max(1, sum(r * k for r, k in zip(rows, ks))), dtype=torch.float64, device=dev)
    S = torch.empty(max(1, sum(ks)), dtype=torch.float64, device=dev)
    V = torch.empty(max(1, sum(c * k for c, k in zip(cols, ks))), dtype=torch.float64, device=dev)
    kept = (C.c_int32 * max(1, nb))()
    spec = (C.c_double * max(1, sum(ks)))()
    slen, terr, dcut = C.c_int32(), C.c_double(), C.c_double()
    try:
        h.call("nd_bs_svd_f64", nb, i64arr(rows), i64arr(cols), i64arr(T.offsets), C.c_void_p(T.data.data_ptr()),
               C.c_void_p(U.data_ptr()), C.c_void_p(S.data_ptr()), C.c_void_p(V.data_ptr()),
               int(_opt(mindim, 1)), int(_opt(maxdim, -1)), float(_opt(cutoff, -1.0)),
               int(bool(use_absolute_cutoff)) if use_absolute_cutoff is not None else 0,
               int(bool(use_relative_cutoff)) if use_relative_cutoff is not None else 1,
               int(_opt(min_blockdim, 0)), kept, spec, C.byref(slen), C.byref(terr), C.byref(dcut))
    except NoConvergence:
        return None
    kept = list(kept[:nb])
    surv = [n for n in range(nb) if kept[n] > 0]
    kdims = [kept[n] for n in surv]
    # new indices u, v: one block per surviving block (linearalgebra.jl:124-156)
    u_ind = tuple(kdims)
    Ublocks = [(T.blocks[n][0], i + 1) for i, n in enumerate(surv)]
    Vblocks = [(T.blocks[n][1], i + 1) for i, n in enumerate(surv)]
    Uo, nu = blockoffsets(Ublocks, [T.inds[0], u_ind])
    Vo, nv = blockoffsets(Vblocks, [T.inds[1], u_ind])
    Ut = BlockSparseTensor([tuple(T.inds[0]), u_ind], Ublocks, Uo, U[:nu])
    Vt = BlockSparseTensor([tuple(T.inds[1]), u_ind], Vblocks, Vo, V[:nv])
    Sv, o = [], 0
    for k in kdims:
        Sv.append(S[o:o + k])
        o += k
    sp = np.array(spec[:slen.value])          # sorted s^2, computed on the device
    return Ut, Sv, Vt, Spectrum(sp, terr.value), kept


class SvdPlan:
    """Blockwise truncated SVD for a fixed block structure whose run() only enqueues
    work on the device, so it can be captured into a CUDA graph (for example with the
    Lanczos loop of a sweep step).  nd_bs_svd_plan_* in the library; the result is the
    one svd() returns (NDTensors/src/blocksparse/linearalgebra.jl:45-215), with kept
    dimensions, spectrum, truncation error and convergence left on the device until
    result() reads them.  Truncation parameters are fixed at construction."""

    def __init__(self, T: BlockSparseTensor, mindim=None, maxdim=None, cutoff=None, use_absolute_cutoff=None,
                 use_relative_cutoff=None, min_blockdim=None):
        import torch
        self.rows, self.cols = _matrix_blocks(T)
        self.nb = len(T.blocks)
        self.blocks = [tuple(b) for b in T.blocks]
        self.inds = [tuple(i) for i in T.inds]
        self.dev = T.data.device
        self.h = handle(self.dev.index or 0)
        self.ptr = C.c_void_p()
        self.h.call("nd_bs_svd_plan_create", self.nb, i64arr(self.rows), i64arr(self.cols), C.byref(self.ptr))
        from ._lib import _live_plans
        _live_plans.add(self)                   # destroyed before the handle at exit
        ks = [min(r, c) for r, c in zip(self.rows, self.cols)]
        f64 = dict(dtype=torch.float64, device=self.dev)
        i32 = dict(dtype=torch.int32, device=self.dev)
        self.U = torch.empty(max(1, sum(r * k for r, k in zip(self.rows, ks))), **f64)
        self.S = torch.empty(max(1, sum(ks)), **f64)
        self.V = torch.empty(max(1, sum(c * k for c, k in zip(self.cols, ks))), **f64)
        self.kept = torch.zeros(max(1, self.nb), **i32)
        self.spectrum = torch.zeros(max(1, sum(ks)), **f64)
        self.slen = torch.zeros(1, **i32)
        self.truncerr = torch.zeros(1, **f64)
        self.status = torch.zeros(1, **i32)
        self.params = (int(_opt(mindim, 1)), int(_opt(maxdim, -1)), float(_opt(cutoff, -1.0)),
                       int(bool(use_absolute_cutoff)) if use_absolute_cutoff is not None else 0,
                       int(bool(use_relative_cutoff)) if use_relative_cutoff is not None else 1,
                       int(_opt(min_blockdim, 0)))

    def run(self, T: BlockSparseTensor):
        """Enqueue the SVD of T (the plan's block structure, any data)."""
        if [tuple(b) for b in T.blocks] != self.blocks:
            raise ValueError("SvdPlan.run: block structure differs from the plan's")
        P = lambda t: C.c_void_p(t.data_ptr())
        handle(self.dev.index or 0)          # bind the handle to torch's current stream
        self.h._check(self.h.lib.nd_bs_svd_plan_exec(
            self.ptr, i64arr(T.offsets), P(T.data), P(self.U), P(self.S), P(self.V), *self.params, P(self.kept),
            P(self.spectrum), P(self.slen), P(self.truncerr), P(self.status)))

    def result(self):
        """(U, S, V, Spectrum, kept) as svd() returns them, or None if a block did not
        converge (reads the device results: synchronises)."""
        if int(self.status.item()) == ND_ERR_NOCONV:
            return None
        kept = self.kept.cpu().tolist()[:self.nb]
        surv = [n for n in range(self.nb) if kept[n] > 0]
        kdims = [kept[n] for n in surv]
        u_ind = tuple(kdims)
        Ublocks = [(self.blocks[n][0], i + 1) for i, n in enumerate(surv)]
        Vblocks = [(self.blocks[n][1], i + 1) for i, n in enumerate(surv)]
        Uo, nu = blockoffsets(Ublocks, [self.inds[0], u_ind])
        Vo, nv = blockoffsets(Vblocks, [self.inds[1], u_ind])
        Ut = BlockSparseTensor([self.inds[0], u_ind], Ublocks, Uo, self.U[:nu])
        Vt = BlockSparseTensor([self.inds[1], u_ind], Vblocks, Vo, self.V[:nv])
        Sv, o = [], 0
        for k in kdims:
            Sv.append(self.S[o:o + k])
            o += k
        n = int(self.slen.item())
        sp = self.spectrum[:n].cpu().numpy()
        return Ut, Sv, Vt, Spectrum(sp, float(self.truncerr.item())), kept

    def destroy(self):
        if self.ptr and self.h.ptr:             # the handle owns the plan's stream and pool
            self.h.lib.nd_bs_svd_plan_destroy(self.ptr)
        self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def eigen(T: BlockSparseTensor, mindim=None, maxdim=None, cutoff=None, use_absolute_cutoff=None,
          use_relative_cutoff=None, min_blockdim=None):
    """Blockwise eigendecomposition of a Hermitian (real symmetric) block-diagonal matrix
    (NDTensors/src/blocksparse/linearalgebra.jl:221-348), one library call
    (nd_bs_eigen_f64): per block the eigenpairs sorted by |lambda| descending, the pooled
    |lambda| sorted and truncated by truncate! and the kept dimension of every block,
    all on the device.

    Returns (D, V, Spectrum, kept): D a list of per-block eigenvalues (truncated), V with
    inds (T.inds[1], v) and one block per surviving block, Spectrum of the pooled |lambda|
    after truncate!; None if a block did not converge (the reference returns nothing).
    """
    import torch
    rows, cols = _matrix_blocks(T)
    for b, r, c in zip(T.blocks, rows, cols):
        if b[0] != b[1] or r != c:
            raise ValueError("eigen: only block-diagonal matrices with square blocks are supported")
    nb = len(T.blocks)
    dev = T.data.device
    Dfull = torch.empty(max(1, sum(rows)), dtype=torch.float64, device=dev)
    Vfull = torch.empty(max(1, sum(r * r for r in rows)), dtype=torch.float64, device=dev)
    kept = (C.c_int32 * max(1, nb))()
    spec = (C.c_double * max(1, sum(rows)))()
    slen, terr, dcut = C.c_int32(), C.c_double(), C.c_double()
    h = handle(dev.index or 0)
    try:
        h.call("nd_bs_eigen_f64", nb, i64arr(rows), i64arr(T.offsets), C.c_void_p(T.data.data_ptr()),
               C.c_void_p(Dfull.data_ptr()), C.c_void_p(Vfull.data_ptr()),
               int(_opt(mindim, 1)), int(_opt(maxdim, -1)), float(_opt(cutoff, -1.0)),
               int(bool(use_absolute_cutoff)) if use_absolute_cutoff is not None else 0,
               int(bool(use_relative_cutoff)) if use_relative_cutoff is not None else 1,
               int(_opt(min_blockdim, 0)), kept, spec, C.byref(slen), C.byref(terr), C.byref(dcut))
    except NoConvergence:
        return None
    kept = list(kept[:nb])
    surv = [n for n in range(nb) if kept[n] > 0]
    v_ind = tuple(kept[n] for n in surv)
    Vblocks = [(T.blocks[n][0], i + 1) for i, n in enumerate(surv)]
    Vo, nv = blockoffsets(Vblocks, [T.inds[1], v_ind])
    D, o = [], 0
    for n in surv:
        D.append(Dfull[o:o + kept[n]])
        o += kept[n]
    Vt = BlockSparseTensor([tuple(T.inds[1]), v_ind], Vblocks, Vo, Vfull[:nv])
    return D, Vt, Spectrum(np.array(spec[:slen.value]), terr.value), kept


def qr(T: BlockSparseTensor, positive=False):
    """Q with inds (T.inds[0], q), R with inds (q, T.inds[1]); q has one block per nz block."""
    import torch
    rows, cols = _matrix_blocks(T)
    nb = len(T.blocks)
    ks = [min(r, c) for r, c in zip(rows, cols)]
    dev = T.data.device
    Q = torch.empty(max(1, sum(r * k for r, k in zip(rows, ks))), dtype=torch.float64, device=dev)
    R = torch.empty(max(1, sum(c * k for c, k in zip(cols, ks))), dtype=torch.float64, device=dev)
    h = handle(T.data.device.index or 0)
    h.call("nd_bs_qr_f64", nb, i64arr(rows), i64arr(cols), i64arr(T.offsets), C.c_void_p(T.data.data_ptr()),
           C.c_void_p(Q.data_ptr()), C.c_void_p(R.data_ptr()), 1 if positive else 0)
    q_ind = tuple(ks)
    Qb = [(T.blocks[n][0], n + 1) for n in range(nb)]
    Rb = [(n + 1, T.blocks[n][1]) for n in range(nb)]
    Qo, nq = blockoffsets(Qb, [T.inds[0], q_ind])
    Ro, nr = blockoffsets(Rb, [q_ind, T.inds[1]])
    return (BlockSparseTensor([tuple(T.inds[0]), q_ind], Qb, Qo, Q[:nq]),
            BlockSparseTensor([q_ind, tuple(T.inds[1])], Rb, Ro, R[:nr]))


def truncate(P, mindim=None, maxdim=None, cutoff=None, use_absolute_cutoff=None, use_relative_cutoff=None):
    """truncate! of a device vector of descending weights -> (new length, truncerr, docut)."""
    h = handle(P.device.index or 0)
    n, te, dc = C.c_int32(), C.c_double(), C.c_double()
    h.call("nd_truncate_f64", C.c_void_p(P.data_ptr()), int(P.numel()), int(_opt(mindim, 1)), int(_opt(maxdim, -1)),
           float(_opt(cutoff, -1.0)), int(bool(use_absolute_cutoff)) if use_absolute_cutoff is not None else 0,
           int(bool(use_relative_cutoff)) if use_relative_cutoff is not None else 1, C.byref(n), C.byref(te),
           C.byref(dc))
    return n.value, te.value, dc.value


# ---------------------------------------------------------------------------
# QN combiner: fuse a group of indices (host structure, device data motion)
# ---------------------------------------------------------------------------

def fused_sectors(group):
    """Sectors of the fused index of [(sectors, arrow), ...], first index fastest
    (src/qn/qnindex.jl:359-379; outer over several indices folds pairwise).  The
    fused arrow is Out unless all arrows agree; charges are arrow*sum(a_k q_k)."""
    arrows = [a for _, a in group]
    arrow = arrows[0] if all(a == arrows[0] for a in arrows) else 1
    out = []
    for combo in itertools.product(*[range(len(s)) for s, _ in reversed(group)]):
        combo = tuple(reversed(combo))
        q = sum(a * s[i][0] for (s, a), i in zip(group, combo))
        d = 1
        for (s, _), i in zip(group, combo):
            d *= s[i][1]
        out.append((arrow * q, d))
    return out, arrow


def combine_blocks(sectors):
    """(combined sectors, perm, comb): stable sort by charge then merge (qnindex.jl:407-426)."""
    perm = sorted(range(len(sectors)), key=lambda i: sectors[i][0])
    comb, merged = [], []
    for pos, i in enumerate(perm):
        if pos > 0 and sectors[i][0] == sectors[perm[pos - 1]][0]:
            merged[-1][1] += sectors[i][1]
        else:
            merged.append([sectors[i][0], sectors[i][1]])
        comb.append(len(merged))
    return [tuple(m) for m in merged], perm, comb


def _group_place(group):
    fused, _ = fused_sectors(group)
    merged, perm, comb = combine_blocks(fused)
    place = {}
    for pos, orig in enumerate(perm):
        off = sum(fused[perm[q]][1] for q in range(pos) if comb[q] == comb[pos])
        place[orig] = (comb[pos], off)          # orig is 0-based fused position
    return merged, place


def _matricize_layout(T: BlockSparseTensor, qinds, row_dims, col_dims):
    """Structure of T fused into (row group, column group) as ITensor's svd / qr do with
    two combiners (src/tensor_operations/matrix_decomposition.jl:153-160), and the block
    copies that fill it: (inds, blocks, offsets, nnz, copies, row_info, col_info)."""
    rows_g = [qinds[d] for d in row_dims]
    cols_g = [qinds[d] for d in col_dims]
    rsec, rplace = _group_place(rows_g)
    csec, cplace = _group_place(cols_g)
    nbr = [len(qinds[d][0]) for d in row_dims]
    nbc = [len(qinds[d][0]) for d in col_dims]

    def lin(b, dims, nbs):
        v, mul = 0, 1
        for d, n in zip(dims, nbs):
            v += (b[d] - 1) * mul
            mul *= n
        return v

    entries = {}
    for i, b in enumerate(T.blocks):
        rb, roff = rplace[lin(b, row_dims, nbr)]
        cb, coff = cplace[lin(b, col_dims, nbc)]
        entries.setdefault((rb, cb), []).append((i, roff, coff))
    mblocks = sorted(entries, key=lambda x: (x[1], x[0]))       # isblockless: column block most significant
    minds = [tuple(d for _, d in rsec), tuple(d for _, d in csec)]
    offs, nnz = blockoffsets(mblocks, minds)
    copies = []
    for j, mb in enumerate(mblocks):
        ld = minds[0][mb[0] - 1]
        for (i, roff, coff) in entries[mb]:
            bd = T.blockdims(T.blocks[i])
            st = [1]
            for d in bd[:-1]:
                st.append(st[-1] * d)
            c = BlockCopy()
            c.src_off = T.offsets[i]
            c.dst_off = offs[j] + roff + coff * ld
            c.rank = len(bd)
            # destination strides: row dims fastest inside the fused row index, then columns (times ld)
            rs, cs = 1, ld
            dst = [0] * len(bd)
            for d in row_dims:
                dst[d] = rs
                rs *= bd[d]
            for d in col_dims:
                dst[d] = cs
                cs *= bd[d]
            for k in range(len(bd)):
                c.dims[k] = bd[k]
                c.src_strides[k] = st[k]
                c.dst_strides[k] = dst[k]
            copies.append(c)
    return minds, mblocks, offs, nnz, copies, (rsec, rplace), (csec, cplace)


def matricize(T: BlockSparseTensor, qinds, row_dims, col_dims):
    """Fuse T's dimensions into (row group, column group) as ITensor's svd / qr do
    with two combiners (src/tensor_operations/matrix_decomposition.jl:153-160).
    qinds: per dimension (sectors, arrow).  Returns (matrix, row_info, col_info)."""
    import torch
    minds, mblocks, offs, nnz, copies, rinfo, cinfo = _matricize_layout(T, qinds, row_dims, col_dims)
    data = torch.zeros(max(nnz, 1), dtype=torch.float64, device=T.data.device)[:nnz]
    M = BlockSparseTensor(minds, mblocks, offs, data)
    if copies:
        arr = (BlockCopy * len(copies))(*copies)
        handle(T.data.device.index or 0).call("nd_block_copy_f64", len(copies), arr, C.c_void_p(T.data.data_ptr()),
                                              C.c_void_p(data.data_ptr()))
    return M, rinfo, cinfo


class MatricizePlan:
    """matricize() for a fixed block structure, prepared once (nd_block_copy_plan_*): run()
    zeroes the matrix and launches the copies, nothing else, so it can be captured into
    a CUDA graph.  The matrix is self.M (its data buffer is reused by every run)."""

    def __init__(self, T: BlockSparseTensor, qinds, row_dims, col_dims):
        import torch
        minds, mblocks, offs, nnz, copies, self.row_info, self.col_info = _matricize_layout(T, qinds, row_dims,
                                                                                           col_dims)
        self.dev = T.data.device
        self.h = handle(self.dev.index or 0)
        self.nnz = nnz
        self.M = BlockSparseTensor(minds, mblocks, offs,
                                   torch.empty(max(nnz, 1), dtype=torch.float64, device=self.dev)[:nnz])
        self.ptr = C.c_void_p()
        arr = (BlockCopy * max(1, len(copies)))(*copies)
        self.h.call("nd_block_copy_plan_create", len(copies), arr, C.byref(self.ptr))
        from ._lib import _live_plans
        _live_plans.add(self)                   # destroyed before the handle at exit

    def run(self, data):
        """self.M <- the matricisation of T's structure on `data` (a flat device vector)."""
        handle(self.dev.index or 0)
        self.h.call("nd_memset0", C.c_void_p(self.M.data.data_ptr()), 8 * self.nnz)
        self.h._check(self.h.lib.nd_block_copy_plan_run(self.ptr, C.c_void_p(data.data_ptr()),
                                                        C.c_void_p(self.M.data.data_ptr())))
        return self.M

    def destroy(self):
        if self.ptr and self.h.ptr:
            self.h.lib.nd_block_copy_plan_destroy(self.ptr)
        self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def uncombine(T: BlockSparseTensor, combdim, group, info, front=False):
    """Split the fused dimension ``combdim`` of T back into the indices of ``group``
    (NDTensors/src/blocksparse/blocksparsetensor.jl:693-791: uncombine_output +
    uncombine, with uncombine_blocks :664-678).

    ``group``: the (sectors, arrow) of the fused indices, in fusion order; ``info``:
    the (combined sectors, place) that ``matricize`` returned for that group.  Every
    block of T, in T's order, yields one block per uncombined sector of its combined
    sector, in the combined index's sorted order (the reference's block order); the
    sub-block is the slice [off, off + dim) of T's block along ``combdim``, copied on
    the device (nd_block_copy_f64) into its own column-major block.  With ``front``
    the uncombined indices come first and the others follow in T's order, as in the
    uncombining contraction with a combiner (NDTensors/src/blocksparse/combiner.jl:90-140,
    which moves the combined index to the front before splitting it; block order is
    unchanged by that move).
    """
    import torch
    _, place = info
    subs = {}
    for orig, (cb, off) in place.items():
        subs.setdefault(cb, []).append((off, orig))
    for v in subs.values():
        v.sort()
    gdims = [tuple(d for _, d in sec) for sec, _ in group]
    nbs = [len(d) for d in gdims]
    if T.rank - 1 + len(gdims) > MAX_RANK:
        raise ValueError(f"uncombine: result rank exceeds {MAX_RANK}")

    def split(lin0):
        out = []
        for n in nbs:
            out.append(lin0 % n + 1)
            lin0 //= n
        return tuple(out)

    others = list(T.inds[:combdim]) + list(T.inds[combdim + 1:])
    inds = gdims + others if front else list(T.inds[:combdim]) + gdims + list(T.inds[combdim + 1:])
    blocks, pieces = [], []
    for i, b in enumerate(T.blocks):
        for off, orig in subs[b[combdim]]:
            if front:
                blocks.append(split(orig) + tuple(b[:combdim]) + tuple(b[combdim + 1:]))
            else:
                blocks.append(tuple(b[:combdim]) + split(orig) + tuple(b[combdim + 1:]))
            pieces.append((i, off))
    offs, nnz = blockoffsets(blocks, inds)
    data = torch.empty(max(nnz, 1), dtype=torch.float64, device=T.data.device)[:nnz]
    R = BlockSparseTensor([tuple(x) for x in inds], blocks, offs, data)
    copies = []
    ng = len(gdims)
    for j, (i, off) in enumerate(pieces):
        tb = T.blockdims(T.blocks[i])
        tst = [1]
        for d in tb[:-1]:
            tst.append(tst[-1] * d)
        rb = R.blockdims(blocks[j])
        c = BlockCopy()
        c.src_off = T.offsets[i] + off * tst[combdim]
        c.dst_off = offs[j]
        c.rank = len(rb)
        gpos = 0 if front else combdim           # where the group's dims sit in the result
        gsrc = []
        g = tst[combdim]
        for k in range(ng):                      # the fused dimension splits first index fastest
            gsrc.append(g)
            g *= rb[gpos + k]
        rest = list(tst[:combdim]) + list(tst[combdim + 1:])
        src = gsrc + rest if front else list(tst[:combdim]) + gsrc + list(tst[combdim + 1:])
        dst = 1
        for k in range(len(rb)):
            c.dims[k] = rb[k]
            c.src_strides[k] = src[k]
            c.dst_strides[k] = dst
            dst *= rb[k]
        copies.append(c)
    if copies:
        arr = (BlockCopy * len(copies))(*copies)
        handle(T.data.device.index or 0).call("nd_block_copy_f64", len(copies), arr, C.c_void_p(T.data.data_ptr()),
                                              C.c_void_p(data.data_ptr()))
    return R


# ---------------------------------------------------------------------------
# Contraction with a combiner (NDTensors/src/blocksparse/combiner.jl:25-143)
# ---------------------------------------------------------------------------

class CombinerTensor:
    """combiner(inds...): fuses QN indices into one combined index whose sectors are
    the fused products (first index fastest), stably sorted by charge and merged
    (src/qn/qnindex.jl:359-426; blockperm / blockcomb of NDTensors' Combiner).

    ``group``: the uncombined indices as (sectors, arrow), in the combiner's order; by
    the reference's convention the combined index is the combiner's first label."""

    def __init__(self, group):
        self.group = [(tuple((int(q), int(d)) for q, d in sec), int(a)) for sec, a in group]
        if not self.group:
            raise ValueError("combiner: no indices to combine")
        merged, self.place = _group_place(self.group)
        self.csec = tuple(tuple(m) for m in merged)
        self.arrow = fused_sectors(self.group)[1]

    @property
    def info(self):
        """(combined sectors, place) as matricize returns it for a group."""
        return (self.csec, self.place)

    @property
    def combined_dims(self):
        return tuple(d for _, d in self.csec)


def _combine_layout(T, fuse_dims, cmb):
    """Host structure of the combining contraction: (inds, blocks, offsets, nnz, copies)
    with one block copy per block of T (see ``combine``)."""
    fuse_dims = [int(d) for d in fuse_dims]
    if len(fuse_dims) != len(cmb.group) or len(set(fuse_dims)) != len(fuse_dims):
        raise ValueError("combine: one distinct tensor dimension per combiner index")
    for d, (sec, _) in zip(fuse_dims, cmb.group):
        if not 0 <= d < T.rank or tuple(T.inds[d]) != tuple(x for _, x in sec):
            raise ValueError(f"combine: dimension {d} does not match the combiner's index")
    rest = [d for d in range(T.rank) if d not in fuse_dims]
    nbs = [len(sec) for sec, _ in cmb.group]
    entries = {}
    for i, b in enumerate(T.blocks):
        lin, mul = 0, 1
        for d, n in zip(fuse_dims, nbs):
            lin += (b[d] - 1) * mul
            mul *= n
        cb, off = cmb.place[lin]
        entries.setdefault((cb,) + tuple(b[d] for d in rest), []).append((i, off))
    cblocks = sorted(entries, key=lambda x: tuple(reversed(x)))    # isblockless
    inds = [cmb.combined_dims] + [tuple(T.inds[d]) for d in rest]
    offs, nnz = blockoffsets(cblocks, inds)
    copies = []
    for j, kb in enumerate(cblocks):
        ld = inds[0][kb[0] - 1]
        for (i, off) in entries[kb]:
            bd = T.blockdims(T.blocks[i])
            c = BlockCopy()
            c.src_off = T.offsets[i]
            c.dst_off = offs[j] + off
            c.rank = len(bd)
            st, dst = 1, [0] * len(bd)
            for d in fuse_dims:                  # inside the combined dimension, combiner order
                dst[d] = st
                st *= bd[d]
            st = ld
            for d in rest:
                dst[d] = st
                st *= bd[d]
            s = 1
            for k in range(len(bd)):
                c.dims[k] = bd[k]
                c.src_strides[k] = s
                c.dst_strides[k] = dst[k]
                s *= bd[k]
            copies.append(c)
    return inds, cblocks, offs, nnz, copies


def combine(T: BlockSparseTensor, fuse_dims, cmb: CombinerTensor):
    """The combining contraction: T's dimensions ``fuse_dims`` (0-based, in the
    combiner's order) become the combined index, placed first, the other dimensions
    follow in T's order (NDTensors/src/blocksparse/combiner.jl:25-89 with
    permutedims_combine_output / permutedims_combine, blocksparsetensor.jl:537-638).

    Output blocks are the combined coordinates ordered by isblockless (last dimension
    most significant) without repeats, offsets in that order; every block of T is
    permuted into its place inside its combined block by one device block copy.
    (Sorting the combined coordinates equals the reference's sort of the sorted-position
    coordinates followed by the merge, since the merge map is non-decreasing.)"""
    import torch
    inds, cblocks, offs, nnz, copies = _combine_layout(T, fuse_dims, cmb)
    data = torch.empty(max(nnz, 1), dtype=torch.float64, device=T.data.device)[:nnz]
    R = BlockSparseTensor(inds, cblocks, offs, data)
    if copies:
        arr = (BlockCopy * len(copies))(*copies)
        handle(T.data.device.index or 0).call("nd_block_copy_f64", len(copies), arr, C.c_void_p(T.data.data_ptr()),
                                              C.c_void_p(data.data_ptr()))
    return R


def contract_combiner(T: BlockSparseTensor, labelsT, Cmb: CombinerTensor, labelsC, labelsR=None,
                      combiner_first=False):
    """contract(T, labelsT, combiner, labelsC) (NDTensors/src/blocksparse/combiner.jl:25-143).

    Combining when the combined label (``labelsC[0]``) is not among T's labels: the
    combiner's other labels must all be T's, and the result is (combined index, T's
    other indices in order).  Uncombining when it is: the result is (the combiner's
    uncombined indices, T's other indices in order).  ``labelsR``, when given, permutes
    that result (block-sparse permutedims).  Dense storage follows the dense rules
    (``_contract_combiner_dense``; ``combiner_first``: the combiner was the call's first
    operand).  Returns (tensor, its labels)."""
    from .contract import permutedims_blocksparse
    from .tensors import DenseTensor
    lt, lc = tuple(labelsT), tuple(labelsC)
    if len(lc) != len(Cmb.group) + 1 or len(lt) != T.rank:
        raise ValueError("combiner contraction: label counts do not match the tensors")
    clabel, uc = lc[0], lc[1:]
    if isinstance(T, DenseTensor):
        return _contract_combiner_dense(T, lt, Cmb, clabel, uc, labelsR, combiner_first)
    if clabel not in lt:
        if any(l not in lt for l in uc):
            raise ValueError("combiner contraction: every uncombined label must be one of the tensor's")
        R = combine(T, [lt.index(l) for l in uc], Cmb)
        out = (clabel,) + tuple(l for l in lt if l not in uc)
    else:
        if any(l in lt for l in uc):
            raise ValueError("combiner contraction: uncombined labels already present on the tensor")
        cpos = lt.index(clabel)
        if tuple(T.inds[cpos]) != Cmb.combined_dims:
            raise ValueError("combiner contraction: the tensor's combined dimension does not match the combiner")
        R = uncombine(T, cpos, Cmb.group, Cmb.info, front=True)
        out = tuple(uc) + tuple(l for l in lt if l != clabel)
    if labelsR is not None and tuple(labelsR) != out:
        lr = tuple(labelsR)
        if sorted(lr) != sorted(out):
            raise ValueError("combiner contraction: output labels do not match")
        R = permutedims_blocksparse(R, [out.index(l) + 1 for l in lr])
        out = lr
    return R, out


def _contract_combiner_dense(T, lt, Cmb, clabel, uc, labelsR, combiner_first):
    """Dense storage (NDTensors/src/combiner/contract.jl:14-77): the output labels follow
    contract_labels of the call (the tensor's free labels, then the combiner's) unless
    ``labelsR`` is given.  Combining permutes the uncombined dimensions together, in the
    combiner's order, to the combined label's place (one device permute) and reshapes;
    uncombining is a reshape of a copy, the uncombined labels taking the combined
    label's place, then a permute if ``labelsR`` asks for another order."""
    from .contract import permutedims
    from .tensors import DenseTensor
    gd = [sum(d for _, d in sec) for sec, _ in Cmb.group]
    if clabel not in lt:
        if any(l not in lt for l in uc):
            raise ValueError("combiner contraction: every uncombined label must be one of the tensor's")
        for l, d in zip(uc, gd):
            if T.dims[lt.index(l)] != d:
                raise ValueError("combiner contraction: a dimension does not match the combiner's index")
        free = tuple(l for l in lt if l not in uc)
        natural = (clabel,) + free if combiner_first else free + (clabel,)
        out = natural if labelsR is None else tuple(labelsR)
        if sorted(out) != sorted(natural):
            raise ValueError("combiner contraction: output labels do not match")
        expanded = []
        for l in out:
            expanded.extend(uc if l == clabel else (l,))
        P = permutedims(T, [lt.index(l) + 1 for l in expanded])
        dims = tuple(int(np.prod(gd)) if l == clabel else T.dims[lt.index(l)] for l in out)
        return DenseTensor(dims, P.data), out
    cpos = lt.index(clabel)
    if any(l in lt for l in uc):
        raise ValueError("combiner contraction: uncombined labels already present on the tensor")
    if T.dims[cpos] != int(np.prod(gd)):
        raise ValueError("combiner contraction: the tensor's combined dimension does not match the combiner")
    natural = lt[:cpos] + tuple(uc) + lt[cpos + 1:]
    dims = tuple(T.dims[:cpos]) + tuple(gd) + tuple(T.dims[cpos + 1:])
    R = DenseTensor(dims, T.data.clone())
    if labelsR is None or tuple(labelsR) == natural:
        return R, natural
    lr = tuple(labelsR)
    if sorted(lr) != sorted(natural):
        raise ValueError("combiner contraction: output labels do not match")
    return permutedims(R, [natural.index(l) + 1 for l in lr]), lr
