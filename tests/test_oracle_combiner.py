"""Contraction with a combiner: the oracle and the host-side layout (CPU).

The oracle's ``combine`` / ``uncombine_front`` restate the reference's combining and
uncombining contraction (NDTensors/src/blocksparse/combiner.jl:25-143 with
permutedims_combine, blocksparsetensor.jl:537-638).  They are pinned here by
  - the reference's own BlockSparse * Combiner test (NDTensors/test/test_combiner.jl:69-101):
    one block (i, j, k) of dims 2 combined over (j, k) gives a (c, i) tensor whose
    permutation (i, c) holds the input's elements in the same linear order, and
    uncombining followed by the permutation (3, 1, 2) gives the input back;
  - a dense reconstruction of the combined index on random QN tensors (sectors of the
    fused product, first index fastest, sorted stably by charge and merged);
  - the round trip combine -> uncombine_front == permutedims.
The library mirror's host layout (block list, offsets and the device block copies,
replayed here on the host) must equal the oracle's result exactly.
"""
import itertools

import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import qn


def _idx(rng, tag, nq, arrow=1):
    return qn.QNIndex(tuple((q, int(rng.integers(1, 4))) for q in range(-nq, nq + 1)), arrow, tag)


def _random_case(seed):
    rng = np.random.default_rng(seed)
    rank = int(rng.integers(3, 6))
    inds = [_idx(rng, f"i{k}", int(rng.integers(1, 3)), int(rng.choice([1, -1]))) for k in range(rank)]
    t = obs.random_blocksparse(rng, [x.dims for x in inds], qn.nzblocks(0, inds))
    nfuse = int(rng.integers(1, min(3, rank - 1) + 1))
    fuse_dims = [int(d) for d in rng.permutation(rank)[:nfuse]]
    return t, inds, fuse_dims


def test_reference_blocksparse_combiner_kat():
    d = 2
    one = qn.QNIndex(((0, d),), 1, "x")
    inds = [one, one, one]
    rng = np.random.default_rng(0)
    t = obs.random_blocksparse(rng, [x.dims for x in inds], [(1, 1, 1)])
    r, info = obs.combine(t, inds, [1, 2])              # contract(T, (1,-1,-2), C, (2,-1,-2))
    assert r.inds == [(d * d,), (d,)]                     # (c, i)
    rp = obs.permutedims(r, (2, 1))
    np.testing.assert_array_equal(rp.data, t.data)        # input_tensor[i] == output_tensor[i]
    back = obs.uncombine_front(rp, 1, [one.dims, one.dims], info)   # contract(out, (1,-1), C, (-1,2,3))
    back = obs.permutedims(back, (3, 1, 2))
    np.testing.assert_array_equal(back.to_dense(), t.to_dense())


@pytest.mark.parametrize("seed", range(8))
def test_combine_dense_reconstruction(seed):
    t, inds, fuse_dims = _random_case(seed)
    r, _ = obs.combine(t, inds, fuse_dims)
    rest = [d for d in range(t.rank) if d not in fuse_dims]
    D = np.transpose(t.to_dense(), fuse_dims + rest)
    group = [inds[d] for d in fuse_dims]
    fused, csec, place = obs.combiner_group(group)
    starts = [np.cumsum((0,) + g.dims) for g in group]

    def colmajor(shape):
        for x in itertools.product(*[range(n) for n in reversed(shape)]):
            yield x[::-1]

    blocks_of = {}                                        # fused product block (1-based) -> its elements
    for orig, combo in enumerate(colmajor([g.nblocks for g in group])):
        shape = [group[k].dims[combo[k]] for k in range(len(group))]
        blocks_of[orig + 1] = [tuple(int(starts[k][combo[k]]) + x[k] for k in range(len(group)))
                               for x in colmajor(shape)]
    flat = [e for o in sorted(blocks_of, key=lambda o: place[o]) for e in blocks_of[o]]
    M = np.stack([D[e] for e in flat])
    assert M.shape[0] == sum(d for _, d in csec)
    np.testing.assert_array_equal(M, r.to_dense().reshape(M.shape))


@pytest.mark.parametrize("seed", range(8))
def test_combine_uncombine_round_trip(seed):
    t, inds, fuse_dims = _random_case(seed)
    r, info = obs.combine(t, inds, fuse_dims)
    back = obs.uncombine_front(r, 0, [inds[d].dims for d in fuse_dims], info)
    rest = [d for d in range(t.rank) if d not in fuse_dims]
    np.testing.assert_array_equal(back.to_dense(), np.transpose(t.to_dense(), fuse_dims + rest))
    # uncombining a combined index that is not first moves it to the front first
    if r.rank > 1:
        rp = obs.permutedims(r, list(range(2, r.rank + 1)) + [1])
        back2 = obs.uncombine_front(rp, r.rank - 1, [inds[d].dims for d in fuse_dims], info)
        np.testing.assert_array_equal(back2.to_dense(), back.to_dense())


def _replay(copies, src, n):
    """Apply the library's block copies on the host."""
    out = np.full(n, np.nan)
    for c in copies:
        dims = [c.dims[k] for k in range(c.rank)]
        for idx in itertools.product(*[range(x) for x in dims]):
            so = c.src_off + sum(i * c.src_strides[k] for k, i in enumerate(idx))
            do = c.dst_off + sum(i * c.dst_strides[k] for k, i in enumerate(idx))
            out[do] = src[so]
    return out


@pytest.mark.parametrize("seed", range(6))
def test_mirror_combine_layout_matches_oracle(seed):
    from ndtensors_gb300.linalg import CombinerTensor, _combine_layout
    from ndtensors_gb300.tensors import BlockSparseTensor
    t, inds, fuse_dims = _random_case(seed)
    ref, (csec, place) = obs.combine(t, inds, fuse_dims)
    cmb = CombinerTensor([(inds[d].sectors, inds[d].arrow) for d in fuse_dims])
    assert cmb.csec == tuple(csec)
    assert {k + 1: v for k, v in cmb.place.items()} == place
    T = BlockSparseTensor([tuple(i) for i in t.inds], list(t.blocks), list(t.offsets), None)
    rinds, blocks, offs, nnz, copies = _combine_layout(T, fuse_dims, cmb)
    assert [tuple(i) for i in rinds] == [tuple(i) for i in ref.inds]
    assert blocks == ref.blocks and offs == ref.offsets and nnz == ref.nnz
    np.testing.assert_array_equal(_replay(copies, t.data, nnz), ref.data)
