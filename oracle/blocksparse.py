"""Block-sparse storage and contraction (oracle restatement).

Storage follows NDTensors: one flat data vector plus an insertion-ordered map
block -> 0-based offset; each block is a dense column-major array of
``prod(blockdims)`` elements (NDTensors/src/blocksparse/blocksparse.jl:5-13,
blockoffsets.jl:11,70-79).  Blocks are 1-based tuples (block.jl:5-16).

Follows:
  NDTensors/src/blocksparse/contract.jl:3-55              contract / contraction_output
  NDTensors/src/blocksparse/contract_sequential.jl:1-41   sequential block plan (bit-exact order)
  NDTensors/src/blocksparse/contract_utilities.jl:28-91   label maps, block matching, blockR
  NDTensors/src/blocksparse/contract_generic.jl:37-129    grouped execution, beta = 0 then 1
  NDTensors/src/blocksparse/blockoffsets.jl:103-111       permutedims of block offsets
  NDTensors/src/blocksparse/blocksparsetensor.jl:834-881  permutedims! per block
  NDTensors/src/blocksparse/blocksparsetensor.jl:537-638  permutedims_combine (matricization)
  NDTensors/src/blocksparse/combiner.jl:25-143            contraction with a combiner
  NDTensors/src/blocksparse/blocksparsetensor.jl:664-791  uncombine
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .dense import contract as dense_contract
from .labels import check_labels, contract_labels, find_matching_positions


def _bdims(inds, block):
    return tuple(inds[k][block[k] - 1] for k in range(len(inds)))


@dataclass
class BlockSparseTensor:
    """inds: list (per dimension) of block-dim tuples; blocks: list of 1-based tuples."""
    inds: list
    blocks: list
    offsets: list
    data: np.ndarray

    @property
    def rank(self):
        return len(self.inds)

    @property
    def nnz(self):
        return int(sum(np.prod(_bdims(self.inds, b)) for b in self.blocks))

    def blockdims(self, block):
        return _bdims(self.inds, block)

    def block_index(self, block):
        return self.blocks.index(tuple(block))

    def blockview(self, i):
        b = self.blocks[i]
        d = self.blockdims(b)
        n = int(np.prod(d)) if d else 1
        off = self.offsets[i]
        return self.data[off:off + n].reshape(d, order="F")

    def to_dense(self):
        full = np.zeros([sum(ix) for ix in self.inds])
        for i, b in enumerate(self.blocks):
            sl = []
            for k, bk in enumerate(b):
                start = sum(self.inds[k][:bk - 1])
                sl.append(slice(start, start + self.inds[k][bk - 1]))
            full[tuple(sl)] = self.blockview(i)
        return full


def blockoffsets(blocks, inds):
    """Offsets in list order (blockoffsets.jl:70-79)."""
    offs, nnz = [], 0
    for b in blocks:
        offs.append(nnz)
        nnz += int(np.prod(_bdims(inds, b)))
    return offs, nnz


def random_blocksparse(rng, inds, blocks):
    offs, nnz = blockoffsets(blocks, inds)
    return BlockSparseTensor(list(map(tuple, inds)), [tuple(b) for b in blocks], offs,
                             rng.standard_normal(nnz))


def are_blocks_contracted(b1, b2, l1_to_l2):
    """contract_utilities.jl:57-70."""
    for i1, i2 in enumerate(l1_to_l2):
        if i2 > 0 and b1[i1] != b2[i2 - 1]:
            return False
    return True


def contract_blocks(b1, l1_to_lr, b2, l2_to_lr, nr):
    """contract_utilities.jl:72-91."""
    br = [0] * nr
    for i1, ir in enumerate(l1_to_lr):
        if ir > 0:
            br[ir - 1] = b1[i1]
    for i2, ir in enumerate(l2_to_lr):
        if ir > 0:
            br[ir - 1] = b2[i2]
    return tuple(br)


def contract_inds_dims(inds1, l1, inds2, l2, lr):
    out = []
    for l in lr:
        out.append(inds1[l1.index(l)] if l in l1 else inds2[l2.index(l)])
    return out


def contract_blockoffsets(t1, l1, t2, l2, lr):
    """Sequential plan: (blocksR, offsetsR, nnzR, plan) with plan entries
    (i1, i2, iR) as 0-based indices into the block lists
    (contract_sequential.jl:1-41)."""
    l1_to_l2 = find_matching_positions(l1, l2)
    l1_to_lr = find_matching_positions(l1, lr)
    l2_to_lr = find_matching_positions(l2, lr)
    indsr = contract_inds_dims(t1.inds, l1, t2.inds, l2, lr)
    blocks_r, offs_r, index_r = [], [], {}
    nnz_r = 0
    plan = []
    for i1, b1 in enumerate(t1.blocks):
        for i2, b2 in enumerate(t2.blocks):
            if are_blocks_contracted(b1, b2, l1_to_l2):
                br = contract_blocks(b1, l1_to_lr, b2, l2_to_lr, len(lr))
                if br not in index_r:
                    index_r[br] = len(blocks_r)
                    blocks_r.append(br)
                    offs_r.append(nnz_r)
                    nnz_r += int(np.prod(_bdims(indsr, br))) if br else 1
                plan.append((i1, i2, index_r[br]))
    return indsr, blocks_r, offs_r, nnz_r, plan


def contract(t1, l1, t2, l2, lr=None, alpha=1.0):
    """Block-sparse contract (contract.jl:3-17 + contract_generic.jl:37-129).

    Pairs are grouped by output block in output-block order; within a group the
    first pair overwrites (beta = 0) and the rest accumulate (beta = 1).
    """
    l1, l2 = tuple(l1), tuple(l2)
    if lr is None:
        lr = contract_labels(l1, l2)
    lr = tuple(lr)
    check_labels(l1, l2, lr)
    indsr, blocks_r, offs_r, nnz_r, plan = contract_blockoffsets(t1, l1, t2, l2, lr)
    r = BlockSparseTensor(indsr, blocks_r, offs_r, np.empty(nnz_r))
    groups = [[] for _ in blocks_r]
    for p in plan:
        groups[p[2]].append(p)
    for g in groups:
        beta = 0.0
        for (i1, i2, ir) in g:
            rv = r.blockview(ir)
            dense_contract(t1.blockview(i1), l1, t2.blockview(i2), l2, lr, alpha=alpha,
                           beta=beta, r=rv)
            beta = 1.0
    return r, plan


def permutedims(t, perm1):
    """Block-sparse permutedims (blockoffsets.jl:103-111, blocksparsetensor.jl:465-470,834-881).

    Blocks keep their order; block coordinates and dims are permuted and the
    offsets are recomputed in that order.
    """
    p0 = [p - 1 for p in perm1]
    inds = [t.inds[k] for k in p0]
    blocks = [tuple(b[k] for k in p0) for b in t.blocks]
    offs, nnz = blockoffsets(blocks, inds)
    r = BlockSparseTensor(inds, blocks, offs, np.empty(nnz))
    for i in range(len(blocks)):
        r.blockview(i)[...] = np.transpose(t.blockview(i), p0)
    return r


def flops_of_plan(t1, l1, t2, l2, plan):
    """Algorithmic flops: sum over pairs of 2*M*N*K."""
    tot = 0
    for (i1, i2, _) in plan:
        d1 = t1.blockdims(t1.blocks[i1])
        d2 = t2.blockdims(t2.blocks[i2])
        m = int(np.prod([d for d, l in zip(d1, l1) if l > 0]))
        k = int(np.prod([d for d, l in zip(d1, l1) if l < 0]))
        n = int(np.prod([d for d, l in zip(d2, l2) if l > 0]))
        tot += 2 * m * n * k
    return tot


# --------------------------------------------------------------------------
# Combiner matricization (blocksparsetensor.jl:537-638, qnindex.jl:407-426)
# --------------------------------------------------------------------------

def _colmajor_linear(block_sub, nblocks_sub):
    """LinearIndices(nblocks)[block...] (1-based), first dimension fastest."""
    lin, mul = 0, 1
    for b, n in zip(block_sub, nblocks_sub):
        lin += (b - 1) * mul
        mul *= n
    return lin + 1


def _isblockless_key(b):
    """isblockless = CartesianIndex ordering: last dimension most significant
    (blockoffsets.jl:35-37)."""
    return tuple(reversed(b))


def combiner_group(idx):
    """The combined index of combiner(idx...) (src/qn/qnindex.jl:359-426): the fused
    index (first index fastest), its sectors stably sorted by charge and merged
    (combineblocks), and for every fused product block (1-based) its (combined block,
    offset inside it), sub-blocks placed in sorted order.  Returns (fused, csec, place)."""
    from .qn import combineblocks, fuse
    fused = fuse(list(idx))
    csec, perm, comb = combineblocks(fused.sectors)
    place = {}
    for pos, orig in enumerate(perm):             # pos: sorted position (0-based), orig: 1-based
        cb = comb[pos]
        off = 0
        q = pos - 1
        while q >= 0 and comb[q] == cb:
            off += fused.sectors[perm[q] - 1][1]
            q -= 1
        place[orig] = (cb, off)
    return fused, csec, place


def matricize(t, qinds, row_dims, col_dims):
    """Fuse a QN block-sparse tensor into a 2-index block matrix.

    Reproduces the structure ITensor's ``svd``/``qr`` build with two combiners
    (src/tensor_operations/matrix_decomposition.jl:153-160): the row group and the
    column group are each fused (first index fastest), their sectors are stably
    sorted by charge and merged (combineblocks), and sub-blocks are placed at
    consecutive offsets inside the merged block in sorted order.  The resulting
    block list is ordered by isblockless (column block most significant).

    ``qinds``: list of oracle.qn.QNIndex for every dimension of ``t``.
    Returns (BlockSparseTensor matrix, row_info, col_info) where *_info holds the
    combined sectors (charge, dim) plus, for every original block-combination of
    the group, its (combined block, offset inside it).
    """
    rfused, rsec, rplace = combiner_group([qinds[d] for d in row_dims])
    cfused, csec, cplace = combiner_group([qinds[d] for d in col_dims])
    nb_rows = [qinds[d].nblocks for d in row_dims]
    nb_cols = [qinds[d].nblocks for d in col_dims]
    entries = {}
    for i, b in enumerate(t.blocks):
        lr_ = _colmajor_linear([b[d] for d in row_dims], nb_rows)
        lc_ = _colmajor_linear([b[d] for d in col_dims], nb_cols)
        rb, roff = rplace[lr_]
        cb, coff = cplace[lc_]
        entries.setdefault((rb, cb), []).append((i, roff, coff))
    mblocks = sorted(entries.keys(), key=_isblockless_key)
    minds = [tuple(d for _, d in rsec), tuple(d for _, d in csec)]
    offs, nnz = blockoffsets(mblocks, minds)
    m = BlockSparseTensor(minds, mblocks, offs, np.zeros(nnz))
    for j, mb in enumerate(mblocks):
        view = m.blockview(j)
        for (i, roff, coff) in entries[mb]:
            blk = t.blockview(i)
            bd = blk.shape
            rdim = int(np.prod([bd[d] for d in row_dims]))
            cdim = int(np.prod([bd[d] for d in col_dims]))
            mat = np.transpose(blk, list(row_dims) + list(col_dims)).reshape(
                (rdim, cdim), order="F")
            view[roff:roff + rdim, coff:coff + cdim] = mat
    return m, (rsec, rplace), (csec, cplace)


def uncombine(t, combdim, group_dims, group_info):
    """Split the fused dimension ``combdim`` of ``t`` back into the indices of its group.

    Restates ``uncombine_output`` / ``uncombine`` (blocksparsetensor.jl:693-791, with
    ``uncombine_blocks`` :664-678 and ``perm_blocks`` :510-517): every block of ``t``,
    in ``t``'s block order, yields one block per uncombined sector of its combined
    sector, in the combined index's sorted order; the sorted position is mapped back
    to the fused product block through the combiner's permutation, and the fused
    block number is split into the group's block numbers column-major (first index
    fastest, ``reshape(::Block, indsT, indsR)``).  The data of sub-block j is the
    slice [off_j, off_j + dim_j) of the combined block along ``combdim``, reshaped.

    ``group_dims``: per group index, its tuple of sector dims (uncombined, original
    order).  ``group_info``: (combined sectors, place) as returned by ``matricize``
    for that group, place[orig] = (combined block, offset) with orig the 1-based
    fused product block.
    """
    _, place = group_info
    subs = {}
    for orig, (cb, off) in place.items():
        subs.setdefault(cb, []).append((off, orig))
    for v in subs.values():
        v.sort()
    nbs = [len(d) for d in group_dims]

    def split(lin0):
        out = []
        for n in nbs:
            out.append(lin0 % n + 1)
            lin0 //= n
        return tuple(out)

    inds = list(t.inds[:combdim]) + [tuple(d) for d in group_dims] + list(t.inds[combdim + 1:])
    blocks, pieces = [], []
    for i, b in enumerate(t.blocks):
        for off, orig in subs[b[combdim]]:
            sub = split(orig - 1)
            blocks.append(tuple(b[:combdim]) + sub + tuple(b[combdim + 1:]))
            pieces.append((i, off))
    offs, nnz = blockoffsets(blocks, inds)
    r = BlockSparseTensor(inds, blocks, offs, np.empty(nnz))
    for j, (i, off) in enumerate(pieces):
        dst = r.blockview(j)
        gsize = int(np.prod([dst.shape[combdim + k] for k in range(len(group_dims))]))
        src = t.blockview(i)
        sl = [slice(None)] * t.rank
        sl[combdim] = slice(off, off + gsize)
        dst[...] = src[tuple(sl)].reshape(dst.shape, order="F")
    return r


# --------------------------------------------------------------------------
# Contraction with a combiner (NDTensors/src/blocksparse/combiner.jl:25-143)
# --------------------------------------------------------------------------

def combine(t, qinds, fuse_dims):
    """contract(T, labels, combiner, labels) in the combining case
    (NDTensors/src/blocksparse/combiner.jl:25-89): the indices ``fuse_dims`` of ``t``
    (0-based, in the combiner's order) become one combined index, placed first, and the
    other indices follow in ``t``'s order.  Restates permutedims_combine_output /
    permutedims_combine (blocksparsetensor.jl:537-638) step by step: permute the block
    coordinates, combine the fused coordinates column-major (combine_dims :487-507),
    map them to sorted positions (perm_blocks :510-517), sort by isblockless, map to
    combined blocks and drop repeats in order (combine_blocks :526-535); then place each
    permuted block at its offset inside the combined block.

    ``qinds``: oracle.qn.QNIndex of every dimension of ``t``.  Returns (tensor, (csec, place)).
    """
    from .qn import combineblocks
    fuse_dims = list(fuse_dims)
    nc = len(fuse_dims)
    rest = [d for d in range(t.rank) if d not in fuse_dims]
    perm = fuse_dims + rest                        # getperm(output_tensor_labels_uc, tensor_labels)
    fused, csec, place = combiner_group([qinds[d] for d in fuse_dims])
    _, blockperm, blockcomb = combineblocks(fused.sectors)
    iperm = [0] * len(blockperm)
    for pos, orig in enumerate(blockperm):
        iperm[orig - 1] = pos + 1
    nbl = [qinds[d].nblocks for d in fuse_dims]

    def perm_comb(b):
        bp = [b[p] for p in perm]
        return (_colmajor_linear(bp[:nc], nbl),) + tuple(bp[nc:])

    blocks = [perm_comb(b) for b in t.blocks]
    blocks = [(iperm[x[0] - 1],) + x[1:] for x in blocks]
    blocks = sorted(blocks, key=_isblockless_key)
    blocks = [(blockcomb[x[0] - 1],) + x[1:] for x in blocks]
    blocks = list(dict.fromkeys(blocks))           # unique!, first occurrences in order
    inds = [tuple(d for _, d in csec)] + [t.inds[d] for d in rest]
    offs, nnz = blockoffsets(blocks, inds)
    r = BlockSparseTensor(inds, blocks, offs, np.zeros(nnz))
    sorted_dims = [fused.sectors[o - 1][1] for o in blockperm]   # permuteblocks(ind_comb, blockperm)
    for i, b in enumerate(t.blocks):
        bpc = perm_comb(b)
        bic = iperm[bpc[0] - 1]                    # b_in_combined_dim (sorted position, 1-based)
        new = blockcomb[bic - 1]
        offset, pos = 0, 1
        while bic - pos > 0 and blockcomb[bic - pos - 1] == new:
            offset += sorted_dims[bic - pos - 1]
            pos += 1
        j = blocks.index((new,) + bpc[1:])
        blk = np.transpose(t.blockview(i), perm)
        dc = sorted_dims[bic - 1]
        sub = blk.reshape((dc,) + blk.shape[nc:], order="F")
        r.blockview(j)[offset:offset + dc, ...] = sub
    return r, (csec, place)


def uncombine_front(t, combdim, group_dims, group_info):
    """contract(T, labels, combiner, labels) in the uncombining case
    (NDTensors/src/blocksparse/combiner.jl:90-140): the combined index (dimension
    ``combdim``) is first moved to the front by a block-sparse permutedims (block order
    kept), then split into the combiner's indices there (``uncombine``), so the result
    is (uncombined indices..., the other indices of ``t`` in order)."""
    perm1 = [combdim + 1] + [d + 1 for d in range(t.rank) if d != combdim]
    tp = permutedims(t, perm1) if combdim != 0 else t
    return uncombine(tp, 0, group_dims, group_info)
