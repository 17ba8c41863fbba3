"""Pin the CPU oracle to the reference's own known-answer tests (CPU only)."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import blocksparse as bs
from oracle import dense, labels, linalg, networks, qn, truncate

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


@pytest.mark.parametrize("case", KATS["truncate"], ids=lambda c: c["src"])
def test_truncate_kats(case):
    P, truncerr, docut = truncate.truncate(case["P"], **case["kwargs"])
    assert (truncerr, docut) == (case["truncerr"], case["docut"])
    assert len(P) == case["len"]


def test_blocksparse_structure_kat():
    k = KATS["blocksparse_structure"]
    blocks = [tuple(b) for b in k["blocks"]]
    offs, nnz = bs.blockoffsets(blocks, k["inds"])
    assert nnz == k["nnz"] and len(blocks) == k["nnzblocks"]
    t = bs.random_blocksparse(np.random.default_rng(0), k["inds"], blocks)
    for key, dims in k["blockdims"].items():
        b = tuple(int(x) for x in key.split(","))
        assert t.blockdims(b) == tuple(dims)


def test_blocksparse_permutedims_kat():
    k = KATS["blocksparse_permutedims"]
    t = bs.random_blocksparse(np.random.default_rng(1), k["inds"], [tuple(b) for b in k["blocks"]])
    tp = bs.permutedims(t, k["perm"])
    for key, dims in k["blockdims_after"].items():
        b = tuple(int(x) for x in key.split(","))
        assert tp.blockdims(b) == tuple(dims)
    assert tp.nnz == k["nnz"]
    np.testing.assert_array_equal(tp.to_dense(), t.to_dense().T)


def test_insert_blocks_nnz_kat():
    k = KATS["insert_blocks_nnz"]
    seq = []
    for n in range(1, len(k["insert_order"]) + 1):
        _, nnz = bs.blockoffsets([tuple(b) for b in k["insert_order"][:n]], k["inds"])
        seq.append(nnz)
    assert seq == k["nnz_sequence"]


def _qidx(secs, arrow=1, tag="x", prime=0):
    return qn.QNIndex(tuple((int(a), int(b)) for a, b in secs), arrow, tag, prime)


def test_qn_contraction_kat():
    k = KATS["qn_contraction"]
    i = _qidx(k["i"], 1, "i")
    j = _qidx(k["j"], 1, "j")
    A_inds = [i, j.dag()]
    B_inds = [j, i.dag().primed()]
    A_blocks = qn.nzblocks(k["A"]["flux"], A_inds)
    B_blocks = qn.nzblocks(k["B"]["flux"], B_inds)
    assert len(A_blocks) == k["A"]["nnzblocks"] and len(B_blocks) == k["B"]["nnzblocks"]
    rng = np.random.default_rng(2)
    A = bs.random_blocksparse(rng, [x.dims for x in A_inds], A_blocks)
    B = bs.random_blocksparse(rng, [x.dims for x in B_inds], B_blocks)
    la, lb = labels.compute_contraction_labels([x.ident() for x in A_inds], [x.ident() for x in B_inds])
    C, plan = bs.contract(A, la, B, lb)
    assert len(C.blocks) == k["C"]["nnzblocks"]
    C_inds = [i, i.dag().primed()]
    assert all(qn.flux(C_inds, b) == k["C"]["flux"] for b in C.blocks)
    np.testing.assert_allclose(C.to_dense(), A.to_dense() @ B.to_dense(), rtol=1e-14, atol=1e-14)


def test_flux_docstring_kat():
    k = KATS["flux_docstring"]
    i = _qidx(k["i"], 1, "i")
    inds = [i, i.primed().dag()]
    for key, f in k["flux"].items():
        b = tuple(int(x) for x in key.split(","))
        assert qn.flux(inds, b) == f


def _doc_tensor(d, rng):
    i1 = _qidx([[0, d], [1, d]], 1, "i1")
    i2 = _qidx([[0, d], [1, d]], 1, "i2")
    inds = [i1.primed(), i2.primed(), i1.dag(), i2.dag()]
    blocks = qn.nzblocks(0, inds)
    return bs.random_blocksparse(rng, [x.dims for x in inds], blocks)


def test_multithreading_doc_kat():
    k = KATS["multithreading_doc"]
    rng = np.random.default_rng(3)
    A = _doc_tensor(k["d"], rng)
    B = _doc_tensor(k["d"], rng)
    la, lb = (1, 2, -1, -2), (-1, -2, 3, 4)      # A' * B contracts A''s (i1', i2') with B's
    C, plan = bs.contract(A, la, B, lb)
    assert len(plan) == k["pairs"]
    assert bs.flops_of_plan(A, la, B, lb, plan) == k["flops"]
    ref = np.einsum("abij,ijcd->abcd", A.to_dense(), B.to_dense())
    np.testing.assert_allclose(C.to_dense(), ref, rtol=1e-12, atol=1e-12)


def test_threaded_no_blocks_kat():
    k = KATS["threaded_no_blocks"]
    inds = [[1, 1], [1, 1]]
    A = bs.random_blocksparse(np.random.default_rng(4), inds, [tuple(k["A_block"])])
    B = bs.random_blocksparse(np.random.default_rng(5), inds, [tuple(k["B_block"])])
    C, plan = bs.contract(A, (1, -1), B, (-1, 2))
    assert len(C.blocks) == k["nnzblocks"] and C.nnz == k["nnz"] and plan == []


def test_threaded_contraction_kat_structure():
    k = KATS["threaded_contraction"]
    i = _qidx([[0, 5], [1, 5]], 1, "i")           # reduced dims, same structure as 500/500
    inds = [i.primed(), i.dag()]
    A = bs.random_blocksparse(np.random.default_rng(6), [x.dims for x in inds], qn.nzblocks(0, inds))
    C, plan = bs.contract(A, (1, -1), A, (-1, 2))
    assert len(plan) == 2 and len(C.blocks) == 2
    np.testing.assert_allclose(C.to_dense(), A.to_dense() @ A.to_dense(), rtol=1e-13)


def test_svd_min_blockdim_kat():
    k = KATS["svd_min_blockdim"]
    i = _qidx(k["i"], 1, "i")
    j = _qidx(k["i"], 1, "j")
    blocks = qn.nzblocks(0, [i, j])
    X = bs.random_blocksparse(np.random.default_rng(7), [i.dims, j.dims], blocks)
    mats = [X.blockview(n) for n in range(len(blocks))]
    out = linalg.svd_blocks(mats, cutoff=k["cutoff"], min_blockdim=k["min_blockdim"])
    for n, m in enumerate(mats):
        full = min(m.shape)
        kept = out["kept"][n]
        assert kept == full or kept >= k["min_blockdim"]


@pytest.mark.parametrize("which", ["labels_noperm", "labels_perm"])
def test_nan_overwrite_kat(which):
    k = KATS["nan_overwrite"]
    rng = np.random.default_rng(8)
    R = np.full(k["R_dims"], np.nan)
    T1 = rng.standard_normal(k["T1_dims"])
    T2 = rng.standard_normal(k["T2_dims"])
    lab = k[which]
    dense.contract_into(R, lab["R"], T1, lab["T1"], T2, lab["T2"])
    assert not np.isnan(R).any()
    exp = T1 * T2[0, 0] if which == "labels_noperm" else np.transpose(T1, (1, 0, 2)) * T2[0, 0]
    np.testing.assert_allclose(R, exp, rtol=1e-15)


def test_sector_recipe_matches_stated_dims():
    # chi = 2048 / 4096 sector lists of the QN workloads
    d2048 = dict(networks.sector_dims(2048))
    assert d2048 == {-8: 8, -7: 18, -6: 37, -5: 68, -4: 112, -3: 166, -2: 219, -1: 259, 0: 274,
                     1: 259, 2: 219, 3: 166, 4: 112, 5: 68, 6: 37, 7: 18, 8: 8}
    assert sum(dict(networks.sector_dims(4096)).values()) == 4096


def test_qn_pair_structure():
    A, B, _ = networks.qn_pair(2048)
    C, plan = bs.contract(A, (1, 2, -1), B, (-1, 3, 4))
    assert (len(A.blocks), len(B.blocks), len(plan), len(C.blocks)) == (32, 32, 62, 62)
    assert bs.flops_of_plan(A, (1, 2, -1), B, (-1, 3, 4), plan) == 661636456


def test_plan_is_first_appearance_ordered():
    # output blocks appear in the order their first pair is met (contract_sequential.jl:33-36)
    rng = np.random.default_rng(9)
    i = _qidx([[q, 2 + abs(q)] for q in range(-2, 3)], 1, "i")
    j = _qidx([[q, 1 + abs(q)] for q in range(-1, 2)], 1, "j")
    A_inds = [i, j, i.dag().primed()]
    B_inds = [i.primed(), j.dag(), i.primed(2)]
    A = bs.random_blocksparse(rng, [x.dims for x in A_inds], qn.nzblocks(0, A_inds))
    B = bs.random_blocksparse(rng, [x.dims for x in B_inds], qn.nzblocks(0, B_inds))
    C, plan = bs.contract(A, (1, 2, -1), B, (-1, 3, 4))
    seen = []
    for (_, _, ir) in plan:
        if ir not in seen:
            seen.append(ir)
    assert seen == list(range(len(C.blocks)))
    ref = np.einsum("abk,kcd->abcd", A.to_dense(), B.to_dense())
    np.testing.assert_allclose(C.to_dense(), ref, rtol=1e-12, atol=1e-12)


def test_matricize_roundtrip():
    net = networks.qn_heff(chi=256, seed=11)
    psi = net["psi"]
    m, rinfo, cinfo = bs.matricize(psi, net["qinds"]["psi"], (0, 1), (2, 3))
    assert len(m.blocks) == 19                   # fused charges q_l + q_s1 in [-9, 9]
    assert np.isclose(np.linalg.norm(m.data), np.linalg.norm(psi.data))
    # flux 0: the fused row charge and the fused column charge cancel
    for (rb, cb) in m.blocks:
        assert rinfo[0][rb - 1][0] + cinfo[0][cb - 1][0] == 0
    # same values as the dense matricization, up to the row/column sector permutation
    dense_psi = psi.to_dense()
    assert np.isclose(np.linalg.norm(m.to_dense()), np.linalg.norm(dense_psi))


def test_adjoint_oracle_matches_finite_differences():
    from oracle.adjoint import contract_pullback
    rng = np.random.default_rng(10)
    x1 = rng.standard_normal((3, 4, 5))
    x2 = rng.standard_normal((5, 4, 2))
    l1, l2, lr = (1, -1, -2), (-2, -1, 3), (1, 3)
    y = dense.contract(x1, l1, x2, l2, lr)
    ybar = rng.standard_normal(y.shape)
    g1, g2 = contract_pullback(x1, l1, x2, l2, lr, ybar)
    f = lambda a, b: float(np.sum(dense.contract(a, l1, b, l2, lr) * ybar))
    h = 1e-6
    for _ in range(5):
        d1 = rng.standard_normal(x1.shape)
        fd = (f(x1 + h * d1, x2) - f(x1 - h * d1, x2)) / (2 * h)
        assert abs(fd - np.sum(g1 * d1)) <= 1e-6 * max(1.0, abs(fd))
        d2 = rng.standard_normal(x2.shape)
        fd = (f(x1, x2 + h * d2) - f(x1, x2 - h * d2)) / (2 * h)
        assert abs(fd - np.sum(g2 * d2)) <= 1e-6 * max(1.0, abs(fd))


def test_package_workloads_match_oracle_generators():
    """Product-side generators (bench inputs) equal the oracle's restatement bit for bit."""
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "itensors.jl_gb300"))
    from ndtensors_gb300 import workloads as wl
    A, B, _ = networks.qn_pair(512)
    pA, pB = wl.qn_pair(512)
    for o, p in ((A, pA), (B, pB)):
        assert [tuple(b) for b in o.blocks] == p.blocks and list(o.offsets) == p.offsets
        np.testing.assert_array_equal(o.data, p.data)
    net, pnet = networks.qn_heff(chi=256, seed=4), wl.qn_heff(chi=256, seed=4)
    for k in ("L", "psi", "W1", "R"):
        assert [tuple(b) for b in net[k].blocks] == pnet[k].blocks
        np.testing.assert_array_equal(net[k].data, pnet[k].data)


def test_uncombine_roundtrip_oracle():
    """Oracle uncombine (blocksparsetensor.jl:693-791) undoes matricize's combiners."""
    net = networks.qn_heff(chi=256, seed=3)
    psi, qi = net["psi"], net["qinds"]["psi"]
    m, rinfo, cinfo = bs.matricize(psi, qi, (0, 1), (2, 3))
    u = bs.uncombine(bs.uncombine(m, 0, [qi[0].dims, qi[1].dims], rinfo), 2, [qi[2].dims, qi[3].dims], cinfo)
    assert sorted(u.blocks) == sorted(psi.blocks) and u.nnz == psi.nnz
    for i, b in enumerate(psi.blocks):
        assert np.array_equal(u.blockview(u.blocks.index(tuple(b))), psi.blockview(i))
