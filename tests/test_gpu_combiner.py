"""Contraction with a combiner on the GPU vs the oracle (GPU).

contract(T, labels, combiner, labels) (NDTensors/src/blocksparse/combiner.jl:25-143):
combining puts the combined index first and T's other indices after it in order;
uncombining moves the combined index to the front and splits it there.  The library's
results (block list, offsets, data) must equal the oracle's restatement exactly (a
combiner only moves data).  The dense case and the reference's invalid-combining
checks follow NDTensors/test/test_combiner.jl:37-65,69-120.
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import qn

pytestmark = pytest.mark.gpu


def _idx(rng, tag, nq, arrow=1):
    return qn.QNIndex(tuple((q, int(rng.integers(1, 5))) for q in range(-nq, nq + 1)), arrow, tag)


def _case(seed):
    rng = np.random.default_rng(seed)
    rank = int(rng.integers(3, 6))
    inds = [_idx(rng, f"i{k}", int(rng.integers(1, 4)), int(rng.choice([1, -1]))) for k in range(rank)]
    t = obs.random_blocksparse(rng, [x.dims for x in inds], qn.nzblocks(0, inds))
    nfuse = int(rng.integers(1, min(3, rank - 1) + 1))
    fuse = [int(d) for d in rng.permutation(rank)[:nfuse]]
    return t, inds, fuse


def _same(nd_t, ref):
    assert [tuple(i) for i in nd_t.inds] == [tuple(i) for i in ref.inds]
    assert list(nd_t.blocks) == list(ref.blocks)
    assert list(nd_t.offsets) == list(ref.offsets)
    np.testing.assert_array_equal(nd_t.data_numpy(), ref.data)


@pytest.mark.parametrize("seed", range(10))
def test_combine_and_uncombine_match_oracle(nd, seed):
    t, inds, fuse = _case(seed)
    T = nd.BlockSparseTensor.from_oracle(t)
    cmb = nd.CombinerTensor([(inds[d].sectors, inds[d].arrow) for d in fuse])
    lt = tuple(range(1, t.rank + 1))
    lc = (100,) + tuple(lt[d] for d in fuse)
    R = nd.contract(T, lt, cmb, lc)
    ref, info = obs.combine(t, inds, fuse)
    _same(R, ref)
    # the combiner as the first operand gives the same block-sparse result
    _same(nd.contract(cmb, lc, T, lt), ref)
    # uncombine with the combined index moved last first: it returns to the front
    rl = (100,) + tuple(l for l in lt if l not in lc[1:])
    perm = list(range(2, ref.rank + 1)) + [1]
    Rp = nd.permutedims_blocksparse(R, perm)
    rpl = tuple(rl[p - 1] for p in perm)
    U = nd.contract(Rp, rpl, cmb, lc)
    refp = obs.permutedims(ref, perm)
    refu = obs.uncombine_front(refp, ref.rank - 1, [inds[d].dims for d in fuse], info)
    _same(U, refu)
    # back to T's label order: the input, bit for bit
    out_labels = lc[1:] + tuple(l for l in rpl if l != 100)
    Ut = nd.contract(Rp, rpl, cmb, lc, lt)
    np.testing.assert_array_equal(obs.BlockSparseTensor(list(Ut.inds), list(Ut.blocks), list(Ut.offsets),
                                                        Ut.data_numpy()).to_dense(), t.to_dense())
    assert len(out_labels) == t.rank


def test_reference_dense_combiner(nd):
    """NDTensors/test/test_combiner.jl:37-65: (d, d, d) combined over the last two
    labels gives (d, d^2) with the same elements in linear order; uncombining restores
    the input; a tensor without the combiner's indices is rejected."""
    d = 2
    rng = np.random.default_rng(3)
    a = rng.standard_normal((d, d, d))
    A = nd.DenseTensor.from_numpy(a)
    cmb = nd.CombinerTensor([(((0, d),), 1), (((0, d),), 1)])
    out = nd.contract(A, (1, -1, -2), cmb, (2, -1, -2))
    assert out.dims == (d, d * d)
    np.testing.assert_array_equal(out.data.cpu().numpy(), A.data.cpu().numpy())
    back = nd.contract(out, (1, -1), cmb, (-1, 2, 3))
    assert back.dims == (d, d, d)
    np.testing.assert_array_equal(back.to_numpy(), a)
    with pytest.raises(ValueError):
        nd.contract(nd.DenseTensor.from_numpy(rng.standard_normal(d)), (-1,), cmb, (1, -1, -2))


def test_dense_combiner_permutes(nd):
    rng = np.random.default_rng(4)
    a = rng.standard_normal((3, 4, 5, 6))
    A = nd.DenseTensor.from_numpy(a)
    cmb = nd.CombinerTensor([(((0, 6),), 1), (((0, 4),), 1)])      # combines labels 4 then 2
    out = nd.contract(A, (1, 2, 3, 4), cmb, (9, 4, 2))
    expect = np.transpose(a, (0, 2, 3, 1)).reshape((3, 5, 24), order="F")   # (1, 3, c) with c = (4, 2)
    np.testing.assert_array_equal(out.to_numpy(), expect)
    first = nd.contract(cmb, (9, 4, 2), A, (1, 2, 3, 4))                 # combiner first: (c, 1, 3)
    np.testing.assert_array_equal(first.to_numpy(), np.transpose(expect, (2, 0, 1)))
    back = nd.contract(out, (1, 3, 9), cmb, (9, 4, 2), (1, 2, 3, 4))
    np.testing.assert_array_equal(back.to_numpy(), a)


def test_blocksparse_invalid_combining(nd):
    """NDTensors/test/test_combiner.jl:103-120: a tensor missing the combiner's indices
    is rejected."""
    t, inds, fuse = _case(1)
    T = nd.BlockSparseTensor.from_oracle(t)
    cmb = nd.CombinerTensor([(inds[d].sectors, inds[d].arrow) for d in fuse])
    with pytest.raises(ValueError):
        nd.contract(T, tuple(range(1, t.rank + 1)), cmb, (100,) + tuple(50 + k for k in range(len(fuse))))
