"""Block-sparse contraction on the GPU vs the oracle (GPU).

Structure (pair list, output blocks, offsets) must be bit-exact with the
reference's sequential plan; values within the precision's tolerance
(relative Frobenius error vs the FP64 oracle): fp64 1e-13, ozaki 1e-10,
bf16x3 1e-4.
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import dense as odense
from oracle import networks, qn

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-13, "ozaki": 1e-10, "bf16x3": 1e-4}


def _q(secs, arrow=1, tag="x", prime=0):
    return qn.QNIndex(tuple((int(a), int(b)) for a, b in secs), arrow, tag, prime)


def _check(nd, A, la, B, lb, lr, precision="fp64"):
    ref, plan = obs.contract(A, la, B, lb, lr)
    GA, GB = nd.BlockSparseTensor.from_oracle(A), nd.BlockSparseTensor.from_oracle(B)
    p = nd.get_plan(GA, la, GB, lb, lr)
    # bit-exact structure
    assert p.pairs == [tuple(x) for x in plan]
    assert p.blocksR == [tuple(b) for b in ref.blocks]
    assert p.offsetsR == list(ref.offsets)
    assert p.nnzR == ref.nnz
    R = nd.contract(GA, la, GB, lb, lr, precision=precision)
    out = R.data_numpy()
    if ref.nnz:
        assert odense.rel_frobenius_error(out, ref.data) <= TOL[precision]
    return p


@pytest.mark.parametrize("precision", ["fp64", "ozaki", "bf16x3"])
def test_qn_pair_workload(nd, precision):
    A, B, _ = networks.qn_pair(2048)
    p = _check(nd, A, (1, 2, -1), B, (-1, 3, 4), (1, 2, 3, 4), precision)
    assert (p.npairs, p.nblocksR) == (62, 62)


def test_multithreading_doc_structure(nd):
    rng = np.random.default_rng(3)
    d = 20
    i1, i2 = _q([[0, d], [1, d]], 1, "i1"), _q([[0, d], [1, d]], 1, "i2")
    inds = [i1.primed(), i2.primed(), i1.dag(), i2.dag()]
    A = obs.random_blocksparse(rng, [x.dims for x in inds], qn.nzblocks(0, inds))
    B = obs.random_blocksparse(rng, [x.dims for x in inds], qn.nzblocks(0, inds))
    for prec in ("fp64", "ozaki"):
        p = _check(nd, A, (1, 2, -1, -2), B, (-1, -2, 3, 4), (1, 2, 3, 4), prec)
        assert p.npairs == 10                       # several pairs per output block


def test_empty_result(nd):
    inds = [[1, 1], [1, 1]]
    A = obs.random_blocksparse(np.random.default_rng(4), inds, [(1, 1)])
    B = obs.random_blocksparse(np.random.default_rng(5), inds, [(2, 2)])
    p = _check(nd, A, (1, -1), B, (-1, 2), (1, 2))
    assert p.npairs == 0 and p.nblocksR == 0 and p.nnzR == 0


@pytest.mark.parametrize("seed", range(6))
def test_random_structures(nd, seed):
    """Random QN tensors, random label placement and output order (permuted blocks)."""
    rng = np.random.default_rng(100 + seed)
    nq = int(rng.integers(2, 5))
    def idx(tag):
        return _q([[q, int(rng.integers(1, 9))] for q in range(-nq, nq + 1)], 1, tag)
    i, j, k, m = idx("i"), idx("j"), idx("k"), idx("m")
    A_inds = [i, k.dag(), j]
    B_inds = [m, k, j.dag()]
    A = obs.random_blocksparse(rng, [x.dims for x in A_inds], qn.nzblocks(int(rng.integers(-1, 2)), A_inds))
    B = obs.random_blocksparse(rng, [x.dims for x in B_inds], qn.nzblocks(0, B_inds))
    la, lb = (1, -1, -2), (2, -1, -2)
    lr = (2, 1) if seed % 2 else (1, 2)
    for prec in ("fp64", "ozaki"):
        _check(nd, A, la, B, lb, lr, prec)


def test_heff_steps_blocksparse(nd):
    net = networks.qn_heff(chi=256, seed=12)
    st = networks.heff_steps()
    t = net["psi"]
    tensors = [(net["L"], st[0], True), (net["W1"], st[1], False), (net["W2"], st[2], False), (net["R"], st[3], False)]
    cur = None
    for (T, (l1, l2, lr), first) in tensors:
        if first:
            ref, _ = obs.contract(T, l1, t, l2, lr)
            _check(nd, T, l1, t, l2, lr, "fp64")
            _check(nd, T, l1, t, l2, lr, "ozaki")
        else:
            ref, _ = obs.contract(cur, l1, T, l2, lr)
            _check(nd, cur, l1, T, l2, lr, "fp64")
            _check(nd, cur, l1, T, l2, lr, "ozaki")
        cur = ref


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_adjoint(nd, precision):
    from oracle.adjoint import contract_pullback
    A, B, _ = networks.qn_pair(256, seed=21)
    la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
    R, plan = obs.contract(A, la, B, lb, lr)
    rng = np.random.default_rng(22)
    Rbar = obs.BlockSparseTensor(R.inds, R.blocks, R.offsets, rng.standard_normal(R.nnz))
    # oracle pullback in dense form, projected on the block structures of A and B
    Ad, Bd, Rbd = A.to_dense(), B.to_dense(), Rbar.to_dense()
    gA, gB = contract_pullback(Ad, (1, 2, 5), Bd, (5, 3, 4), (1, 2, 3, 4), Rbd)
    GA, GB = nd.BlockSparseTensor.from_oracle(A), nd.BlockSparseTensor.from_oracle(B)
    p = nd.get_plan(GA, la, GB, lb, lr)
    import torch
    GR = torch.from_numpy(Rbar.data).cuda()
    Abar = torch.full((A.nnz,), float("nan"), dtype=torch.float64, device="cuda")
    Bbar = torch.full((B.nnz,), float("nan"), dtype=torch.float64, device="cuda")
    import ctypes as C
    from ndtensors_gb300._lib import PRECISIONS
    p.h.call("nd_bs_contract_adjoint_f64", p.ptr, C.c_void_p(GR.data_ptr()), C.c_void_p(GA.data.data_ptr()),
             C.c_void_p(GB.data.data_ptr()), C.c_void_p(Abar.data_ptr()), C.c_void_p(Bbar.data_ptr()),
             PRECISIONS[precision])
    Ab = obs.BlockSparseTensor(A.inds, A.blocks, A.offsets, Abar.cpu().numpy()).to_dense()
    Bb = obs.BlockSparseTensor(B.inds, B.blocks, B.offsets, Bbar.cpu().numpy()).to_dense()
    assert odense.rel_frobenius_error(Ab, gA) <= TOL[precision]
    assert odense.rel_frobenius_error(Bb, gB) <= TOL[precision]


def _plan_structure(nd, GA, la, GB, lb, lr):
    p = nd.ContractionPlan(GA, la, GB, lb, lr)
    s = (p.pairs, p.blocksR, p.offsetsR, p.nnzR)
    p.destroy()
    return s


def _placement_cases():
    """(A, labels A, B, labels B, labels R) covering several shapes of plan."""
    rng = np.random.default_rng(410)
    out = []
    A, B, _ = networks.qn_pair(2048)
    out.append((A, (1, 2, -1), B, (-1, 3, 4), (1, 2, 3, 4)))
    for seed in range(3):
        r = np.random.default_rng(420 + seed)
        nq = 3
        def idx(tag):
            return _q([[q, int(r.integers(1, 6))] for q in range(-nq, nq + 1)], 1, tag)
        i, j, k, m = idx("i"), idx("j"), idx("k"), idx("m")
        A_inds, B_inds = [i, k.dag(), j], [m, k, j.dag()]
        A = obs.random_blocksparse(r, [x.dims for x in A_inds], qn.nzblocks(0, A_inds))
        B = obs.random_blocksparse(r, [x.dims for x in B_inds], qn.nzblocks(0, B_inds))
        out.append((A, (1, -1, -2), B, (2, -1, -2), (2, 1) if seed % 2 else (1, 2)))
    # no contracted index (outer product): every pair matches, 90 x 70 = 6300 pairs, more
    # than the host placement takes by default
    A = obs.random_blocksparse(rng, [(1,) * 90, (2,)], [(a, 1) for a in range(1, 91)])
    B = obs.random_blocksparse(rng, [(1,) * 70], [(b,) for b in range(1, 71)])
    out.append((A, (1, 2), B, (3,), (3, 1, 2)))
    # two contracted indices, B blocks listed out of order, output order swapped
    A = obs.random_blocksparse(rng, [(3, 4), (2, 2, 5), (1, 2)], [(1, 1, 2), (2, 2, 1), (1, 3, 1), (2, 3, 2)])
    B = obs.random_blocksparse(rng, [(2, 2, 5), (1, 2), (6, 2)], [(3, 1, 1), (2, 1, 2), (3, 2, 2), (1, 2, 1)])
    out.append((A, (1, -1, -2), B, (-1, -2, 2), (2, 1)))
    return out


def test_plan_placements_agree(nd):
    """Host planner, device planner and the size-based choice give the reference's plan:
    pairs, output blocks and offsets bit-exact with the oracle in every placement."""
    h = nd.handle(0)
    try:
        for A, la, B, lb, lr in _placement_cases():
            ref, plan = obs.contract(A, la, B, lb, lr)
            want = ([tuple(x) for x in plan], [tuple(b) for b in ref.blocks], list(ref.offsets), ref.nnz)
            GA, GB = nd.BlockSparseTensor.from_oracle(A), nd.BlockSparseTensor.from_oracle(B)
            for where in (2, 1, 0):
                h.call("nd_set_plan_placement", where)
                assert _plan_structure(nd, GA, la, GB, lb, lr) == want, f"placement {where}"
        with pytest.raises(nd.NDError):
            h.call("nd_set_plan_placement", 3)
    finally:
        h.call("nd_set_plan_placement", 0)


def test_plan_rejects_mismatched_blocks(nd):
    A = obs.random_blocksparse(np.random.default_rng(0), [[2, 3], [4, 5]], [(1, 1)])
    B = obs.random_blocksparse(np.random.default_rng(0), [[4, 6], [2]], [(1, 1)])
    with pytest.raises(nd.NDError):
        nd.get_plan(nd.BlockSparseTensor.from_oracle(A), (1, -1), nd.BlockSparseTensor.from_oracle(B), (-1, 2),
                    (1, 2))


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_skinny_group_with_many_pairs(nd, precision):
    """One output block fed by 12 skinny pairs (K = 2 each, N = 3): more pairs than one
    staging round of the skinny kernel holds, operands spread over 2^+-40."""
    rng = np.random.default_rng(9)
    A = obs.random_blocksparse(rng, [(5000,), (2,) * 12], [(1, k) for k in range(1, 13)])
    B = obs.random_blocksparse(rng, [(2,) * 12, (3,)], [(k, 1) for k in range(1, 13)])
    A.data[:] *= 2.0 ** rng.integers(-40, 40, A.data.shape)
    p = _check(nd, A, (1, -1), B, (-1, 2), (1, 2), precision)
    assert (p.npairs, p.nblocksR) == (12, 1)


@pytest.mark.parametrize("rank,seed", [(3, 0), (4, 1), (5, 2), (4, 3)])
def test_bs_permutedims_matches_oracle(nd, rank, seed):
    """Block-sparse permutedims (blocksparsetensor.jl:465-470,834-881; blockoffsets.jl:103-111)
    through nd_bs_permutedims_f64: block list, offsets and data bit-exact with the oracle
    on QN tensors of rank 3-5 with a random permutation."""
    rng = np.random.default_rng(300 + seed)
    inds = [_q([[q, int(rng.integers(1, 7))] for q in range(-2, 3)], int(rng.choice([-1, 1])), f"i{k}")
            for k in range(rank)]
    T = obs.random_blocksparse(rng, [x.dims for x in inds], qn.nzblocks(0, inds))
    assert len(T.blocks) > 4
    perm = tuple(int(p) + 1 for p in rng.permutation(rank))
    ref = obs.permutedims(T, perm)
    R = nd.permutedims_blocksparse(nd.BlockSparseTensor.from_oracle(T), perm)
    assert R.blocks == [tuple(b) for b in ref.blocks]
    assert R.offsets == list(ref.offsets)
    assert [tuple(i) for i in R.inds] == [tuple(i) for i in ref.inds]
    np.testing.assert_array_equal(R.data_numpy(), ref.data)


def test_ozaki_split_k_bit_identical(nd):
    """The split GEMM cuts a long-K tile into K ranges only when the launch's other work is
    small: a 10 x 12 output with K = 30000 is split when contracted alone and not when it
    shares the launch with a 4000^3 block pair.  The ranges start on 512-K chunk
    boundaries and their exact int64 partials are summed before the one conversion, so
    both results must be equal bit for bit (and within 1e-10 of FP64)."""
    rng = np.random.default_rng(77)
    a1, b1 = rng.standard_normal((10, 30000)), rng.standard_normal((30000, 12))
    a2, b2 = rng.standard_normal((4000, 4000)), rng.standard_normal((4000, 4000))
    A = obs.BlockSparseTensor([(10, 4000), (30000, 4000)], [(1, 1), (2, 2)], [0, a1.size],
                              np.concatenate([a1.reshape(-1, order="F"), a2.reshape(-1, order="F")]))
    B = obs.BlockSparseTensor([(30000, 4000), (12, 4000)], [(1, 1), (2, 2)], [0, b1.size],
                              np.concatenate([b1.reshape(-1, order="F"), b2.reshape(-1, order="F")]))
    R = nd.contract(nd.BlockSparseTensor.from_oracle(A), (1, -1), nd.BlockSparseTensor.from_oracle(B), (-1, 2),
                    precision="ozaki")
    i = list(R.blocks).index((1, 1))
    shared = R.data_numpy()[R.offsets[i]:R.offsets[i] + 120]
    alone = nd.DenseTensor.empty((10, 12))
    nd.contract_(alone, (1, 2), nd.DenseTensor.from_numpy(a1), (1, -1), nd.DenseTensor.from_numpy(b1), (-1, 2),
                 1.0, 0.0, "ozaki")
    alone = alone.to_numpy().reshape(-1, order="F")
    np.testing.assert_array_equal(shared, alone)
    assert odense.rel_frobenius_error(alone, (a1 @ b1).reshape(-1, order="F")) <= 1e-10


def test_blocksparse_permutedims_large_and_small_blocks(nd):
    """Blocks of 2^22 elements or more take the tiled transposer, smaller ones the batched
    gather: a tensor with one large block (2048 x 2100) among small ones, permuted, is
    bit-exact with the oracle (structure and data)."""
    rng = np.random.default_rng(404)
    inds = [(2048, 3, 5), (2100, 4, 6)]
    blocks = [(1, 1), (2, 2), (3, 3), (2, 3), (3, 1)]
    T = obs.random_blocksparse(rng, inds, blocks)
    ref = obs.permutedims(T, (2, 1))
    R = nd.permutedims_blocksparse(nd.BlockSparseTensor.from_oracle(T), (2, 1))
    assert R.blocks == [tuple(b) for b in ref.blocks] and R.offsets == list(ref.offsets)
    np.testing.assert_array_equal(R.data_numpy(), ref.data)
