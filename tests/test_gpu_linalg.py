"""Blockwise SVD / QR / truncate! / combiner on the GPU vs the oracle (GPU).

Singular values: within 1e-12 of LAPACK gesdd relative to the block's largest;
reconstruction U S V^T within 1e-12 relative Frobenius; truncation decisions
(kept dims per block, truncerr, spectrum length) identical to the oracle.
"""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import dense as odense
from oracle import linalg as olin
from oracle import networks, qn
from oracle import truncate as otr

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def _gpu(nd, t):
    return nd.BlockSparseTensor.from_oracle(t)


def _blocks(nd, T):
    """Per-block dense numpy matrices of a GPU block-sparse matrix."""
    out = []
    data = T.data_numpy()
    for i, b in enumerate(T.blocks):
        d = T.blockdims(b)
        out.append(data[T.offsets[i]:T.offsets[i] + d[0] * d[1]].reshape(d, order="F"))
    return out


# the five structures of NDTensors/test/test_blocksparse.jl:276-321
SVD_EXAMPLES = [
    ([(2, 1), (1, 2)], [2, 2], [2, 2]),
    ([(1, 2), (2, 3)], [2, 2], [3, 2, 3]),
    ([(2, 1), (3, 2)], [3, 2, 3], [2, 2]),
    ([(2, 1), (3, 2)], [2, 3, 4], [5, 6]),
    ([(1, 2), (2, 3)], [5, 6], [2, 3, 4]),
]


@pytest.mark.parametrize("ex", SVD_EXAMPLES)
def test_svd_reference_examples(nd, ex):
    blocks, i1, i2 = ex
    A = obs.random_blocksparse(np.random.default_rng(1), [i1, i2], blocks)
    U, S, V, spec, kept = nd.svd(_gpu(nd, A))
    Ub, Vb = _blocks(nd, U), _blocks(nd, V)
    for n, m in enumerate(_blocks(nd, _gpu(nd, A))):
        s = S[n].cpu().numpy()
        np.testing.assert_allclose(Ub[n] @ np.diag(s) @ Vb[n].T, m, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(s, np.linalg.svd(m, compute_uv=False), rtol=1e-12, atol=1e-12 * s[0])


@pytest.mark.parametrize("spectrum", ["gaussian", "graded", "clustered"])
def test_svd_preconditioned_blocks(nd, spectrum):
    """Blocks large enough for the FP32-preconditioned path (work >= 2e8): same bars as
    the plain FP64 path, including singular values down to 1e-13 of the largest and
    near-degenerate clusters (which the FP32 phase cannot separate)."""
    rng = np.random.default_rng({"gaussian": 31, "graded": 32, "clustered": 33}[spectrum])
    dims = [(700, 600), (520, 560), (64, 90)]
    mats = []
    for (r, c) in dims:
        k = min(r, c)
        if spectrum == "gaussian":
            m = rng.standard_normal((r, c))
        else:
            if spectrum == "graded":
                sv = np.logspace(0, -13, k)
            else:
                sv = np.repeat(np.linspace(1.0, 0.1, 8), -(-k // 8))[:k] * (1 + 1e-9 * rng.standard_normal(k))
            qu, _ = np.linalg.qr(rng.standard_normal((r, k)))
            qv, _ = np.linalg.qr(rng.standard_normal((c, k)))
            m = (qu * sv) @ qv.T
        mats.append(m)
    inds = [[d[0] for d in dims], [d[1] for d in dims]]
    blocks = [(i + 1, i + 1) for i in range(len(dims))]
    offs, o = [], 0
    for m in mats:
        offs.append(o)
        o += m.size
    A = obs.BlockSparseTensor(inds, blocks, offs, np.concatenate([m.reshape(-1, order="F") for m in mats]))
    U, S, V, spec, kept = nd.svd(_gpu(nd, A))
    Ub, Vb = _blocks(nd, U), _blocks(nd, V)
    for n, m in enumerate(mats):
        s = S[n].cpu().numpy()
        ref = np.linalg.svd(m, compute_uv=False)
        np.testing.assert_allclose(s, ref, rtol=0, atol=1e-12 * ref[0])
        assert odense.rel_frobenius_error(Ub[n] @ np.diag(s) @ Vb[n].T, m) <= 1e-12
        k = len(s)
        np.testing.assert_allclose(Vb[n].T @ Vb[n], np.eye(k), atol=1e-12)


@pytest.mark.parametrize("shape", [(40, 40), (130, 33), (33, 130), (257, 255), (1, 7), (600, 64)])
def test_svd_dense_block(nd, shape):
    rng = np.random.default_rng(sum(shape))
    m = rng.standard_normal(shape)
    A = obs.BlockSparseTensor([[shape[0]], [shape[1]]], [(1, 1)], [0], m.reshape(-1, order="F"))
    U, S, V, spec, kept = nd.svd(_gpu(nd, A))
    u, s, v = _blocks(nd, U)[0], S[0].cpu().numpy(), _blocks(nd, V)[0]
    ref = np.linalg.svd(m, compute_uv=False)
    np.testing.assert_allclose(s, ref, rtol=0, atol=1e-12 * ref[0])
    assert odense.rel_frobenius_error(u @ np.diag(s) @ v.T, m) <= 1e-12
    k = len(s)
    np.testing.assert_allclose(u.T @ u, np.eye(k), atol=1e-12)
    np.testing.assert_allclose(v.T @ v, np.eye(k), atol=1e-12)
    np.testing.assert_allclose(spec.eigs, np.sort(ref ** 2)[::-1], rtol=1e-12, atol=1e-12 * ref[0] ** 2)


def test_svd_graded_spectrum_truncation(nd):
    """Blocks with geometric singular values: truncation by cutoff must match the oracle exactly."""
    rng = np.random.default_rng(5)
    mats = []
    for n, (r, c) in enumerate([(60, 50), (40, 70), (30, 30), (8, 12)]):
        q1, _ = np.linalg.qr(rng.standard_normal((r, r)))
        q2, _ = np.linalg.qr(rng.standard_normal((c, c)))
        k = min(r, c)
        sv = np.exp(-np.arange(k) * (0.35 + 0.1 * n)) * (1.0 + n)
        d = np.zeros((r, c))
        d[:k, :k] = np.diag(sv)
        mats.append(q1 @ d @ q2.T)
    inds = [[m.shape[0] for m in mats], [m.shape[1] for m in mats]]
    blocks = [(i + 1, i + 1) for i in range(len(mats))]
    offs, nnz = obs.blockoffsets(blocks, inds)
    A = obs.BlockSparseTensor(inds, blocks, offs, np.concatenate([m.reshape(-1, order="F") for m in mats]))
    for kw in ({"cutoff": 1e-10}, {"cutoff": 1e-6, "maxdim": 40}, {"maxdim": 25},
               {"cutoff": 1e-8, "use_absolute_cutoff": True}, {"cutoff": 1e-1, "min_blockdim": 2}):
        ref = olin.svd_blocks(mats, **kw)
        U, S, V, spec, kept = nd.svd(_gpu(nd, A), **kw)
        assert kept == ref["kept"], kw
        assert len(spec.eigs) == len(ref["spectrum"])
        np.testing.assert_allclose(spec.eigs, ref["spectrum"], rtol=1e-10, atol=1e-14)
        assert abs(spec.truncerr - ref["truncerr"]) <= 1e-10 * max(1.0, abs(ref["truncerr"])) + 1e-15


@pytest.mark.parametrize("case", KATS["truncate"], ids=lambda c: c["src"])
def test_truncate_kats_on_device(nd, case):
    import torch
    P = torch.tensor(case["P"], dtype=torch.float64, device="cuda")
    n, te, dc = nd.truncate(P, **case["kwargs"])
    assert (te, dc) == (case["truncerr"], case["docut"])
    assert n == case["len"]


def test_svd_min_blockdim_kat(nd):
    k = KATS["svd_min_blockdim"]
    i = qn.QNIndex(tuple(tuple(x) for x in k["i"]), 1, "i")
    j = qn.QNIndex(tuple(tuple(x) for x in k["i"]), 1, "j")
    X = obs.random_blocksparse(np.random.default_rng(7), [i.dims, j.dims], qn.nzblocks(0, [i, j]))
    mats = [X.blockview(n) for n in range(len(X.blocks))]
    ref = olin.svd_blocks(mats, cutoff=k["cutoff"], min_blockdim=k["min_blockdim"])
    U, S, V, spec, kept = nd.svd(_gpu(nd, X), cutoff=k["cutoff"], min_blockdim=k["min_blockdim"])
    assert kept == ref["kept"]
    for n, m in enumerate(mats):
        assert kept[n] == min(m.shape) or kept[n] >= k["min_blockdim"]


@pytest.mark.parametrize("positive", [False, True])
@pytest.mark.parametrize("shape", [(30, 30), (50, 20), (20, 50), (1, 5), (200, 100)])
def test_qr_blocks(nd, shape, positive):
    rng = np.random.default_rng(shape[0] * 7 + shape[1])
    mats = [rng.standard_normal(shape), rng.standard_normal((shape[1], shape[0]))]
    inds = [[shape[0], shape[1]], [shape[1], shape[0]]]
    blocks = [(1, 1), (2, 2)]
    offs, nnz = obs.blockoffsets(blocks, inds)
    A = obs.BlockSparseTensor(inds, blocks, offs, np.concatenate([m.reshape(-1, order="F") for m in mats]))
    Q, R = nd.qr(_gpu(nd, A), positive=positive)
    oq, orr = olin.qr_blocks(mats, positive=positive)
    for n, m in enumerate(mats):
        q, r = _blocks(nd, Q)[n], _blocks(nd, R)[n]
        np.testing.assert_allclose(q @ r, m, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(q.T @ q, np.eye(q.shape[1]), atol=1e-12)
        assert np.allclose(np.tril(r, -1), 0)
        if positive:
            assert (np.diag(r) >= 0).all()
        # same sign convention as LAPACK geqrf (and unique when positive)
        np.testing.assert_allclose(q, oq[n], rtol=1e-10, atol=1e-10)
        np.testing.assert_allclose(r, orr[n], rtol=1e-10, atol=1e-10)


@pytest.mark.parametrize("positive", [False, True])
def test_qr_blocked_panels(nd, positive):
    """Blocks spanning several 32-column panels and partial 16-column strips (tall, wide,
    square, a 1036 x 1036 block as in the chi = 4096 matricisation): Q R = A, Q
    orthonormal, R upper triangular, LAPACK's geqrf signs."""
    rng = np.random.default_rng(91)
    shapes = [(300, 200), (130, 300), (257, 257), (64, 33), (1036, 1036), (5, 1)]
    mats = [rng.standard_normal(sh) for sh in shapes]
    inds = [[sh[0] for sh in shapes], [sh[1] for sh in shapes]]
    blocks = [(i + 1, i + 1) for i in range(len(shapes))]
    offs, nnz = obs.blockoffsets(blocks, inds)
    A = obs.BlockSparseTensor(inds, blocks, offs, np.concatenate([m.reshape(-1, order="F") for m in mats]))
    Q, R = nd.qr(_gpu(nd, A), positive=positive)
    oq, orr = olin.qr_blocks(mats, positive=positive)
    qb, rb = _blocks(nd, Q), _blocks(nd, R)
    for n, m in enumerate(mats):
        q, r = qb[n], rb[n]
        np.testing.assert_allclose(q @ r, m, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(m).max()) * max(m.shape))
        np.testing.assert_allclose(q.T @ q, np.eye(q.shape[1]), atol=1e-12 * max(m.shape))
        assert np.allclose(np.tril(r, -1), 0)
        if positive:
            assert (np.diag(r) >= 0).all()
        np.testing.assert_allclose(q, oq[n], rtol=1e-9, atol=1e-9)
        np.testing.assert_allclose(r, orr[n], rtol=1e-9, atol=1e-9 * max(1.0, np.abs(orr[n]).max()))


def test_matricize_matches_oracle(nd):
    net = networks.qn_heff(chi=256, seed=11)
    psi = net["psi"]
    qinds = net["qinds"]["psi"]
    ref, rinfo, cinfo = obs.matricize(psi, qinds, (0, 1), (2, 3))
    M, _, _ = nd.matricize(_gpu(nd, psi), [(q.sectors, q.arrow) for q in qinds], (0, 1), (2, 3))
    assert M.blocks == [tuple(b) for b in ref.blocks]
    assert M.offsets == list(ref.offsets)
    np.testing.assert_array_equal(M.data_numpy(), ref.data)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_two_site_step(nd, precision):
    """H_eff matvec -> matricize (l,s1)x(s2,r) -> truncated blockwise SVD, vs the oracle."""
    net = networks.qn_heff(chi=512, seed=13)
    steps = networks.heff_steps()
    # oracle
    t, _ = obs.contract(net["L"], steps[0][0], net["psi"], steps[0][1], steps[0][2])
    for (a, b, c), key in zip(steps[1:], ("W1", "W2", "R")):
        t, _ = obs.contract(t, a, net[key], b, c)
    qi = [net["qinds"]["psi"][k] for k in range(4)]          # result has psi's structure (lo, s1o, s2o, ro)
    Mref, _, _ = obs.matricize(t, qi, (0, 1), (2, 3))
    mats = [Mref.blockview(n) for n in range(len(Mref.blocks))]
    ref = olin.svd_blocks(mats, maxdim=512, cutoff=1e-10)
    # GPU
    G = {k: _gpu(nd, net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    x = nd.contract(G["L"], steps[0][0], G["psi"], steps[0][1], steps[0][2], precision=precision)
    for (a, b, c), key in zip(steps[1:], ("W1", "W2", "R")):
        x = nd.contract(x, a, G[key], b, c, precision=precision)
    assert x.blocks == [tuple(b) for b in t.blocks]
    assert odense.rel_frobenius_error(x.data_numpy(), t.data) <= (1e-13 if precision == "fp64" else 1e-10)
    M, _, _ = nd.matricize(x, [(q.sectors, q.arrow) for q in qi], (0, 1), (2, 3))
    U, S, V, spec, kept = nd.svd(M, maxdim=512, cutoff=1e-10)
    assert kept == ref["kept"]
    np.testing.assert_allclose(spec.eigs, ref["spectrum"], rtol=1e-8, atol=1e-13 * ref["spectrum"][0])
    assert abs(spec.truncerr - ref["truncerr"]) <= 1e-8 * ref["truncerr"] + 1e-16


@pytest.mark.parametrize("case", ["full", "truncated", "min_blockdim"])
def test_eigen_blockwise_matches_oracle(nd, case):
    """Blockwise Hermitian eigen (linearalgebra.jl:221-348) vs the oracle (numpy eigh per
    block, |lambda|-sorted, pooled truncate!, per-block kept dims)."""
    rng = np.random.default_rng({"full": 61, "truncated": 62, "min_blockdim": 63}[case])
    dims = [40, 130, 7, 260]
    mats = []
    for n in dims:
        q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        lam = rng.standard_normal(n) * np.exp(rng.uniform(-12, 0, n))     # both signs, wide range
        mats.append((q * lam) @ q.T)
    mats.append(np.zeros((5, 5)))                                          # a zero block
    mats.append(-np.outer(np.ones(6), np.ones(6)))                         # rank one, negative
    dims = [m.shape[0] for m in mats]
    offs, o = [], 0
    for m in mats:
        offs.append(o)
        o += m.size
    A = obs.BlockSparseTensor([dims, dims], [(i + 1, i + 1) for i in range(len(dims))], offs,
                              np.concatenate([m.reshape(-1, order="F") for m in mats]))
    kw = {"full": {}, "truncated": {"maxdim": 150, "cutoff": 1e-9},
          "min_blockdim": {"cutoff": 1e-3, "min_blockdim": 2}}[case]
    ref = olin.eigen_blocks(mats, **kw)
    D, V, spec, kept = nd.eigen(_gpu(nd, A), **kw)
    assert kept == ref["kept"]
    # error scale of lambda = sigma - c with c ~ ||A_b||_F: eps-level multiples of ||A_b||_F
    fro = max(np.linalg.norm(m) for m in mats)
    np.testing.assert_allclose(spec.eigs, ref["spectrum"], rtol=0, atol=1e-12 * fro)
    assert abs(spec.truncerr - ref["truncerr"]) <= 1e-10 * max(ref["truncerr"], 1e-300) + 1e-15
    Vb = _blocks(nd, V)
    surv = [n for n in range(len(mats)) if kept[n] > 0]
    for i, n in enumerate(surv):
        m, lam, vec = mats[n], D[i].cpu().numpy(), Vb[i]
        scale = max(np.linalg.norm(m), 1e-300)
        np.testing.assert_allclose(lam, ref["D"][i], rtol=0, atol=1e-12 * scale)
        np.testing.assert_allclose(vec.T @ vec, np.eye(len(lam)), atol=1e-12)
        np.testing.assert_allclose(m @ vec, vec * lam, rtol=0, atol=1e-11 * scale)   # eigenpairs


@pytest.mark.parametrize("kind", ["psd", "plus_minus_pairs"])
def test_eigen_unshifted_and_fallback_paths(nd, kind):
    """Positive semidefinite blocks (density matrices) take the unshifted path: the SVD of
    the block is its eigendecomposition.  Blocks with exact +-lambda pairs make the
    singular vectors of a pair mix, which the sign check catches, and the shifted path
    decomposes them instead.  Both vs the oracle (numpy eigh)."""
    rng = np.random.default_rng(64 if kind == "psd" else 65)
    mats = []
    for n in (90, 250, 12):
        q, _ = np.linalg.qr(rng.standard_normal((n, n)))
        if kind == "psd":
            lam = np.exp(rng.uniform(-18, 0, n))
        else:
            half = np.exp(rng.uniform(-6, 0, n // 2))
            lam = np.concatenate([half, -half, [0.5]][: 3 if n % 2 else 2])[:n]
        mats.append((q * lam) @ q.T)
    dims = [m.shape[0] for m in mats]
    offs, o = [], 0
    for m in mats:
        offs.append(o)
        o += m.size
    A = obs.BlockSparseTensor([dims, dims], [(i + 1, i + 1) for i in range(len(dims))], offs,
                              np.concatenate([m.reshape(-1, order="F") for m in mats]))
    kw = {"maxdim": 200, "cutoff": 1e-12}
    ref = olin.eigen_blocks(mats, **kw)
    D, V, spec, kept = nd.eigen(_gpu(nd, A), **kw)
    assert kept == ref["kept"]
    Vb = _blocks(nd, V)
    surv = [n for n in range(len(mats)) if kept[n] > 0]
    for i, n in enumerate(surv):
        m, lam, vec = mats[n], D[i].cpu().numpy(), Vb[i]
        scale = np.linalg.norm(m)
        np.testing.assert_allclose(np.sort(np.abs(lam))[::-1], np.sort(np.abs(ref["D"][i]))[::-1], rtol=0,
                                   atol=1e-12 * scale)
        np.testing.assert_allclose(vec.T @ vec, np.eye(len(lam)), atol=1e-12)
        np.testing.assert_allclose(m @ vec, vec * lam, rtol=0, atol=1e-11 * scale)


def test_diag_blocksparse_contraction_rebuilds_svd(nd):
    """BlockSparse x DiagBlockSparse (blocksparse/diagblocksparse.jl:601-696): U * S * V^T
    rebuilt from the blockwise SVD equals the input; the output structure is the plan's
    (contraction_output) and matches the oracle's contraction with the expanded diagonal."""
    import torch
    rng = np.random.default_rng(72)
    dims = [50, 80, 33]
    mats = [rng.standard_normal((d, d + 7)) for d in dims]
    inds = [dims, [d + 7 for d in dims]]
    blocks = [(i + 1, i + 1) for i in range(len(dims))]
    offs, nnz = obs.blockoffsets(blocks, inds)
    A = obs.BlockSparseTensor(inds, blocks, offs, np.concatenate([m.reshape(-1, order="F") for m in mats]))
    U, S, V, spec, kept = nd.svd(_gpu(nd, A))
    u_ind = U.inds[1]
    D = nd.DiagBlockSparseTensor.from_diagonals([u_ind, u_ind], [(i + 1, i + 1) for i in range(len(S))], S)
    US = nd.contract(U, (1, -1), D, (-1, 2))                # diag operand second
    SU = nd.contract(D, (-1, 2), U, (1, -1))                 # diag operand first: labels (1, 2) by default
    assert SU.blocks == US.blocks and SU.offsets == US.offsets
    np.testing.assert_array_equal(SU.data_numpy(), US.data_numpy())
    R = nd.contract(US, (1, -1), V, (2, -1))                 # (l, r)
    out = obs.BlockSparseTensor(R.inds, R.blocks, R.offsets, R.data_numpy()).to_dense()
    assert odense.rel_frobenius_error(out, A.to_dense()) <= 1e-12
    # oracle: the same contraction with the diagonal expanded to dense blocks
    Dd = D.dense()
    Do = obs.BlockSparseTensor([list(u_ind), list(u_ind)], Dd.blocks, Dd.offsets, Dd.data_numpy())
    Uo = obs.BlockSparseTensor([list(U.inds[0]), list(u_ind)], U.blocks, U.offsets, U.data_numpy())
    ref, _ = obs.contract(Uo, (1, -1), Do, (-1, 2), (1, 2))
    assert US.blocks == [tuple(b) for b in ref.blocks] and US.offsets == list(ref.offsets)
    assert odense.rel_frobenius_error(US.data_numpy(), ref.data) <= 1e-14


def test_uncombine_inverts_matricize(nd):
    """combine -> uncombine is the identity up to block order (blocksparsetensor.jl:537-638 and
    :693-791), and the uncombined structure, offsets and data are those of the oracle."""
    net = networks.qn_heff(chi=256, seed=14)
    psi = net["psi"]
    qi = net["qinds"]["psi"]
    qp = [(q.sectors, q.arrow) for q in qi]
    M, rinfo, cinfo = nd.matricize(_gpu(nd, psi), qp, (0, 1), (2, 3))
    rows = nd.uncombine(M, 0, qp[:2], rinfo)                 # (l, s1, (s2 r))
    back = nd.uncombine(rows, 2, qp[2:], cinfo)             # (l, s1, s2, r)
    Mo, orinfo, ocinfo = obs.matricize(psi, qi, (0, 1), (2, 3))
    ro = obs.uncombine(Mo, 0, [qi[0].dims, qi[1].dims], orinfo)
    bo = obs.uncombine(ro, 2, [qi[2].dims, qi[3].dims], ocinfo)
    for got, want in ((rows, ro), (back, bo)):
        assert got.blocks == [tuple(b) for b in want.blocks]
        assert got.offsets == list(want.offsets)
        np.testing.assert_array_equal(got.data_numpy(), want.data)
    data = back.data_numpy()
    assert sorted(back.blocks) == sorted(tuple(b) for b in psi.blocks)
    for i, b in enumerate(psi.blocks):
        j = back.blocks.index(tuple(b))
        n = int(np.prod(psi.blockdims(b)))
        np.testing.assert_array_equal(data[back.offsets[j]:back.offsets[j] + n], psi.data[psi.offsets[i]:psi.offsets[i] + n])


@pytest.mark.parametrize("dims,panel", [
    ([(2000, 320), (120, 90)], 1),     # tall block: FP32 panels of 2 x 8 columns, FP64 panels of 2 x 4
    ([(7000, 20), (30, 30)], 0),       # taller than any shared-memory panel: scalar sweeps
])
def test_svd_panel_widths_and_scalar_fallback(nd, dims, panel):
    """The sweep stage picks the widest column group whose panel fits shared memory and
    falls back to the scalar sweep above that; every path meets the same bars.  The
    convergence record (nd_svd_last_info) reports which one ran."""
    import ctypes as C
    rng = np.random.default_rng(41 + panel)
    mats = [rng.standard_normal(d) for d in dims]
    offs, o = [], 0
    for m in mats:
        offs.append(o)
        o += m.size
    A = obs.BlockSparseTensor([[d[0] for d in dims], [d[1] for d in dims]], [(i + 1, i + 1) for i in range(len(dims))],
                              offs, np.concatenate([m.reshape(-1, order="F") for m in mats]))
    U, S, V, spec, kept = nd.svd(_gpu(nd, A))
    ints = (C.c_int32 * 16)()
    dbls = (C.c_double * 16)()
    nd.handle(0).call("nd_svd_last_info", ints, 16, dbls, 16)
    assert ints[3] == panel and ints[2] >= 1                  # panel flag, FP64 sweeps
    Ub, Vb = _blocks(nd, U), _blocks(nd, V)
    for n, m in enumerate(mats):
        s = S[n].cpu().numpy()
        ref = np.linalg.svd(m, compute_uv=False)
        np.testing.assert_allclose(s, ref, rtol=0, atol=1e-12 * ref[0])
        assert odense.rel_frobenius_error(Ub[n] @ np.diag(s) @ Vb[n].T, m) <= 1e-12
        np.testing.assert_allclose(Vb[n].T @ Vb[n], np.eye(len(s)), atol=1e-12)
        np.testing.assert_allclose(Ub[n].T @ Ub[n], np.eye(len(s)), atol=1e-12)


def test_svd_spectrum_kat(nd):
    """test/base/test_decomp.jl:433-446: the spectrum of A = U diag(S) V' with |S| = 1
    holds S.^2 with no truncation error, and maxdim = length(S) - 3 discards exactly
    the three smallest (truncerror = their sum of squares)."""
    rng = np.random.default_rng(17)
    u, s, vt = np.linalg.svd(rng.random((100, 100)))
    s = s / np.linalg.norm(s)
    a = u @ np.diag(s) @ vt
    A = obs.random_blocksparse(rng, [(100,), (100,)], [(1, 1)])
    A.data[:] = a.reshape(-1, order="F")
    _, _, _, spec, _ = nd.svd(_gpu(nd, A))
    np.testing.assert_allclose(nd.eigs(spec), s ** 2, rtol=1e-10, atol=1e-15)
    assert nd.truncerror(spec) == 0.0
    _, _, _, spec, kept = nd.svd(_gpu(nd, A), maxdim=len(s) - 3)
    assert list(kept) == [len(s) - 3]
    np.testing.assert_allclose(nd.truncerror(spec), np.sum(s[-3:] ** 2), rtol=1e-8)


def test_qn_svd_truncation_invariants(nd):
    """test/base/test_qnitensor.jl:1272-1318 (svd truncation example 1): A(i, j, i', j')
    with i = j = [QN(0) => 2, QN(1) => 3], flux 0, raised to the 16th power as a matrix
    (i, j) x (i', j') and normalised; svd with cutoff 1e-5 must keep fewer than dim(i)
    dim(j) values, one per spectrum entry, with truncerr <= cutoff, and the
    reconstruction's relative error 1 - |Ap|^2 / |A|^2 within rtol 1e-6 of truncerr."""
    rng = np.random.default_rng(23)
    i = qn.QNIndex(((0, 2), (1, 3)), 1, "i")
    j = qn.QNIndex(((0, 2), (1, 3)), 1, "j")
    inds = [i, j, i.dag().primed(), j.dag().primed()]
    t = obs.random_blocksparse(rng, [x.dims for x in inds], qn.nzblocks(0, inds))
    M, _, _ = obs.matricize(t, inds, (0, 1), (2, 3))
    for _ in range(4):                                    # A = mapprime(A * A', 2, 1), four times
        for n in range(len(M.blocks)):
            v = M.blockview(n)
            v[...] = v @ v
    M.data /= np.linalg.norm(M.data)
    cutoff = 1e-5
    U, S, V, spec, kept = nd.svd(_gpu(nd, M), cutoff=cutoff)
    assert sum(kept) == len(spec.eigs) < i.dim * j.dim
    assert spec.truncerr <= cutoff
    ub, vb = _blocks(nd, U), _blocks(nd, V)
    ap2 = sum(float(np.sum((ub[n] @ np.diag(S[n].cpu().numpy()) @ vb[n].T) ** 2)) for n in range(len(ub)))
    err = 1.0 - ap2 / float(np.sum(M.data ** 2))
    assert err <= cutoff
    np.testing.assert_allclose(err, spec.truncerr, rtol=1e-6)
