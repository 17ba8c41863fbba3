"""One two-site sweep update as one CUDA graph (GPU).

SweepStep captures the whole update -- the Lanczos solve of H_eff with its small
tridiagonal problem on the device, the matricisation of the Ritz vector and the
truncated blockwise SVD -- and replays it.  Checked against the host-driven path
(Lanczos with the host eigensolve, matricize, svd) and the oracle on the same Ritz
vector: energy to 1e-12 relative, the Ritz vector up to sign, kept dimensions and the
spectrum identical, truncation error within 1e-10; a second replay from a new start
vector agrees with a fresh eager SweepStep bit for bit.  Also the device tridiagonal
eigensolver against numpy on random matrices.
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import linalg as olin
from oracle import networks

pytestmark = pytest.mark.gpu


def test_tridiag_lowest_matches_eigh(nd):
    import torch
    import ctypes as C
    rng = np.random.default_rng(61)
    h = nd.handle(0)
    P = lambda t: C.c_void_p(t.data_ptr())
    for k in (1, 2, 5, 10, 31, 32):
        a = rng.standard_normal(k) * 3.0
        b = rng.standard_normal(max(k - 1, 1))
        if k == 10:
            b[:] = np.abs(b) * 1e-9                    # nearly diagonal
        T = np.diag(a) + np.diag(b[:k - 1], 1) + np.diag(b[:k - 1], -1)
        w, v = np.linalg.eigh(T)
        ad, bd = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        val, y = torch.zeros(1, dtype=torch.float64, device="cuda"), torch.zeros(k, dtype=torch.float64, device="cuda")
        h.call("nd_tridiag_lowest_f64", k, P(ad), P(bd), P(val), P(y))
        yv = y.cpu().numpy()
        assert abs(val.item() - w[0]) <= 1e-13 * max(1.0, np.abs(w).max())
        assert np.linalg.norm(T @ yv - val.item() * yv) <= 1e-10 * max(1.0, np.abs(w).max())
        assert abs(np.linalg.norm(yv) - 1.0) <= 1e-14


def test_sweep_step_graph(nd):
    import torch
    net = networks.qn_heff(chi=512, seed=62)
    steps = networks.heff_steps()
    G = {k: nd.BlockSparseTensor.from_oracle(net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    psi = G["psi"]
    qi = net["qinds"]["psi"]
    qpairs = [(q.sectors, q.arrow) for q in qi]
    kw = dict(maxdim=400, cutoff=1e-10)
    # host-driven reference path
    op = nd.HeffOperator(G["L"], G["W1"], G["W2"], G["R"], psi, steps, precision="ozaki")
    r = nd.Lanczos(op.apply, op.n, krylovdim=8).run(psi.data)
    # the whole update as one graph
    sw = nd.SweepStep(G["L"], G["W1"], G["W2"], G["R"], psi, steps, qpairs, (0, 1), (2, 3), krylovdim=8,
                      precision="ozaki", graph=True, **kw)
    sw.run(psi.data)
    energy, x, res = sw.result()
    assert abs(energy - r.value) <= 1e-12 * abs(r.value)
    xr = r.vector.cpu().numpy()
    xg = x.cpu().numpy()
    assert abs(abs(xg @ xr) / (np.linalg.norm(xg) * np.linalg.norm(xr)) - 1.0) <= 1e-10
    # the SVD of the graph's Ritz vector vs the oracle on that vector
    host = obs.BlockSparseTensor([tuple(i) for i in psi.inds], [tuple(b) for b in psi.blocks], list(psi.offsets), xg)
    Mref, _, _ = obs.matricize(host, qi, (0, 1), (2, 3))
    np.testing.assert_array_equal(sw.mat.M.data_numpy(), Mref.data)
    mats = [Mref.blockview(n) for n in range(len(Mref.blocks))]
    ref = olin.svd_blocks(mats, **kw)
    U, S, V, spec, kept = res
    assert kept == list(ref["kept"])
    np.testing.assert_allclose(spec.eigs, ref["spectrum"], rtol=1e-10, atol=1e-13 * ref["spectrum"][0])
    assert abs(spec.truncerr - ref["truncerr"]) <= 1e-10
    smax = max(float(s[0]) for s in ref["S"])
    for s_gpu, s_ref in zip(S, ref["S"]):
        np.testing.assert_allclose(s_gpu.cpu().numpy(), s_ref, rtol=0, atol=1e-12 * smax)
    # replay from a new start vector == a fresh eager SweepStep on the same start, bit for bit
    v1 = psi.data.clone()
    v1.add_(torch.linspace(-1e-3, 1e-3, v1.numel(), dtype=torch.float64, device=v1.device))
    sw.run(v1)
    e1, x1, res1 = sw.result()
    got = (e1, x1.cpu().numpy().copy(), res1[0].data_numpy().copy(), res1[2].data_numpy().copy(), list(res1[4]))
    eg = nd.SweepStep(G["L"], G["W1"], G["W2"], G["R"], psi, steps, qpairs, (0, 1), (2, 3), krylovdim=8,
                      precision="ozaki", graph=False, **kw)
    eg.run(v1)
    e2, x2, res2 = eg.result()
    assert e2 == got[0]
    np.testing.assert_array_equal(x2.cpu().numpy(), got[1])
    np.testing.assert_array_equal(res2[0].data_numpy(), got[2])
    np.testing.assert_array_equal(res2[2].data_numpy(), got[3])
    assert list(res2[4]) == got[4]
