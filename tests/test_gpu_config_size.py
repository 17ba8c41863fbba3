"""The benchmark configurations at their full sizes, on the GPU vs the oracle (GPU).

- QN two-site H_eff matvec at chi = 4096 (the headline workload): every one of the
  four block plans (pairs, output blocks, offsets) bit-exact with the reference's
  sequential plan, the FP64 result within 1e-13 and the Ozaki result within 1e-10
  relative Frobenius error of the oracle.
- Dense two-site H_eff apply at chi = 1024 (XXZ MPO): FP64 within 1e-13, Ozaki within
  1e-10, 3xBF16 within 1e-4 of the oracle.
- The sweep step's truncated blockwise SVD at chi = 4096 (Lanczos Ritz vector,
  matricized (l,s1) x (s2,r), maxdim 4096, cutoff 1e-10): kept dimensions identical
  to the oracle's, truncation error within 1e-10 (absolute; it is a sum of discarded
  weights of a unit vector), singular values within 1e-12 of the largest; U and V
  uncombined back onto (l, s1, u) and (s2, r, v) with the reference's block order.
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import dense as odense
from oracle import linalg as olin
from oracle import networks

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-13, "ozaki": 1e-10, "bf16x3": 1e-4}


@pytest.fixture(scope="module")
def heff4096():
    net = networks.qn_heff(chi=4096, seed=3)
    steps = networks.heff_steps()
    outs, plans = [], []
    x = net["L"]
    for (a, b, c), key in zip(steps, ("psi", "W1", "W2", "R")):
        x, plan = obs.contract(x, a, net[key], b, c)
        outs.append(x)
        plans.append(plan)
    return net, steps, outs, plans


def test_qn_heff_chi4096_plans_bit_exact(nd, heff4096):
    import torch
    net, steps, outs, plans = heff4096
    G = {k: nd.BlockSparseTensor.from_oracle(net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    x = G["L"]
    for (a, b, c), key, ref, plan in zip(steps, ("psi", "W1", "W2", "R"), outs, plans):
        p = nd.get_plan(x, a, G[key], b, c)
        assert p.pairs == [tuple(q) for q in plan]
        assert p.blocksR == [tuple(bl) for bl in ref.blocks]
        assert p.offsetsR == list(ref.offsets)
        assert p.nnzR == ref.nnz
        x = nd.BlockSparseTensor(list(p.indsR), list(p.blocksR), list(p.offsetsR),
                                 torch.empty(max(p.nnzR, 1), dtype=torch.float64, device="cuda")[:p.nnzR])
    assert [len(p) for p in plans] == [180, 304, 312, 180]


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_qn_heff_chi4096_values(nd, heff4096, precision):
    net, steps, outs, _ = heff4096
    G = {k: nd.BlockSparseTensor.from_oracle(net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    x = G["L"]
    for (a, b, c), key in zip(steps, ("psi", "W1", "W2", "R")):
        x = nd.contract(x, a, G[key], b, c, precision=precision)
    ref = outs[-1]
    assert x.blocks == [tuple(b) for b in ref.blocks] and x.offsets == list(ref.offsets)
    assert odense.rel_frobenius_error(x.data_numpy(), ref.data) <= TOL[precision]


def test_dense_heff_chi1024_all_precisions(nd):
    net = networks.dense_heff(chi=1024)
    steps = networks.heff_steps()
    ref = net["L"]
    for (a, b, c), key in zip(steps, ("psi", "W1", "W2", "R")):
        ref = odense.contract(ref, a, net[key], b, c)
    G = {k: nd.DenseTensor.from_numpy(net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    for precision in ("fp64", "ozaki", "bf16x3"):
        x = G["L"]
        for (a, b, c), key in zip(steps, ("psi", "W1", "W2", "R")):
            x = nd.contract(x, a, G[key], b, c, precision=precision)
        err = odense.rel_frobenius_error(x.to_numpy(), ref)
        assert err <= TOL[precision], f"{precision}: {err:.3e}"


def test_sweep_step_svd_chi4096(nd, heff4096):
    import torch
    net, steps, _, _ = heff4096
    G = {k: nd.BlockSparseTensor.from_oracle(net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    psi = G["psi"]
    op = nd.HeffOperator(G["L"], G["W1"], G["W2"], G["R"], psi, steps, precision="fp64")
    r = nd.Lanczos(op.apply, op.n, krylovdim=10).run(psi.data)
    qi = net["qinds"]["psi"]
    qpairs = [(q.sectors, q.arrow) for q in qi]
    v = nd.BlockSparseTensor(list(psi.inds), list(psi.blocks), list(psi.offsets), r.vector.contiguous())
    M, rinfo, cinfo = nd.matricize(v, qpairs, (0, 1), (2, 3))
    U, S, V, spec, kept = nd.svd(M, maxdim=4096, cutoff=1e-10)
    # oracle on the same Ritz vector
    host = obs.BlockSparseTensor([tuple(i) for i in psi.inds], [tuple(b) for b in psi.blocks], list(psi.offsets),
                                 r.vector.cpu().numpy())
    Mref, orinfo, ocinfo = obs.matricize(host, qi, (0, 1), (2, 3))
    assert M.blocks == [tuple(b) for b in Mref.blocks]
    np.testing.assert_array_equal(M.data_numpy(), Mref.data)
    mats = [Mref.blockview(n) for n in range(len(Mref.blocks))]
    ref = olin.svd_blocks(mats, maxdim=4096, cutoff=1e-10)
    assert len(mats) == 19
    assert kept == ref["kept"] and 0 < sum(kept) <= 4096
    assert abs(spec.truncerr - ref["truncerr"]) <= 1e-10
    smax = max(float(s[0]) for s in ref["S"])
    for s_gpu, s_ref in zip(S, ref["S"]):
        np.testing.assert_allclose(s_gpu.cpu().numpy(), s_ref, rtol=0, atol=1e-12 * smax)
    # U onto (l, s1, u) and V onto (s2, r, v): structure of the reference's uncombine,
    # values as the oracle's own uncombine of the GPU factors
    Uu = nd.uncombine(U, 0, qpairs[:2], rinfo)
    Vu = nd.uncombine(V, 0, qpairs[2:], cinfo)
    Uo = obs.BlockSparseTensor([tuple(i) for i in U.inds], list(U.blocks), list(U.offsets), U.data_numpy())
    Vo = obs.BlockSparseTensor([tuple(i) for i in V.inds], list(V.blocks), list(V.offsets), V.data_numpy())
    Ur = obs.uncombine(Uo, 0, [qi[0].dims, qi[1].dims], orinfo)
    Vr = obs.uncombine(Vo, 0, [qi[2].dims, qi[3].dims], ocinfo)
    for got, want in ((Uu, Ur), (Vu, Vr)):
        assert got.blocks == [tuple(b) for b in want.blocks]
        assert got.offsets == list(want.offsets)
        np.testing.assert_array_equal(got.data_numpy(), want.data)
    # the truncated two-site tensor rebuilt from (l,s1,u) S (s2,r,v) carries the kept weight
    Sd = torch.cat(S)
    w = float((Sd * Sd).sum())
    assert abs(w + spec.truncerr - 1.0) <= 1e-10
