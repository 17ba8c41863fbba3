"""Blockwise SVD plan (nd_bs_svd_plan_*): the truncated SVD with every decision on the
device, so that an execution can be captured into a CUDA graph (GPU).

- Results vs the oracle (LAPACK gesdd per block + truncate!): singular values within
  1e-12 of the block's largest, U S V^T within 1e-12, U and V orthogonal to 1e-12,
  kept dimensions and spectrum identical, truncation error within 1e-10.
- Both paths of the plan: blocks large enough for the FP32 + refinement stages, and
  small blocks (FP64 sweeps only).
- A CUDA-graph replay on new data equals an eager run on the same data bit for bit.
- Non-convergence is reported on the device (sweep limit 0).
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import dense as odense
from oracle import linalg as olin

pytestmark = pytest.mark.gpu


def _matrix(rng, dims, decay=None):
    mats = []
    for (r, c) in dims:
        if decay is None:
            m = rng.standard_normal((r, c))
        else:
            k = min(r, c)
            qu, _ = np.linalg.qr(rng.standard_normal((r, k)))
            qv, _ = np.linalg.qr(rng.standard_normal((c, k)))
            m = (qu * np.logspace(0, decay, k)) @ qv.T
        mats.append(m)
    offs, o = [], 0
    for m in mats:
        offs.append(o)
        o += m.size
    A = obs.BlockSparseTensor([[d[0] for d in dims], [d[1] for d in dims]], [(i + 1, i + 1) for i in range(len(dims))],
                              offs, np.concatenate([m.reshape(-1, order="F") for m in mats]))
    return A, mats


def _dense_blocks(T):
    out = []
    data = T.data_numpy()
    for i, b in enumerate(T.blocks):
        d = T.blockdims(b)
        out.append(data[T.offsets[i]:T.offsets[i] + d[0] * d[1]].reshape(d, order="F"))
    return out


def _check(res, mats, kw):
    U, S, V, spec, kept = res
    ref = olin.svd_blocks(mats, **kw)
    assert kept == list(ref["kept"])
    np.testing.assert_allclose(spec.eigs, ref["spectrum"], rtol=1e-10, atol=1e-13 * ref["spectrum"][0])
    assert abs(spec.truncerr - ref["truncerr"]) <= 1e-10 * max(1.0, abs(ref["truncerr"]))
    Ub, Vb = _dense_blocks(U), _dense_blocks(V)
    surv = [n for n in range(len(mats)) if kept[n] > 0]
    for j, n in enumerate(surv):
        s = S[j].cpu().numpy()
        full = np.linalg.svd(mats[n], compute_uv=False)
        np.testing.assert_allclose(s, full[:len(s)], rtol=0, atol=1e-12 * full[0])
        np.testing.assert_allclose(Ub[j].T @ Ub[j], np.eye(len(s)), atol=1e-12)
        np.testing.assert_allclose(Vb[j].T @ Vb[j], np.eye(len(s)), atol=1e-12)
        if len(s) == min(mats[n].shape):
            assert odense.rel_frobenius_error(Ub[j] @ np.diag(s) @ Vb[j].T, mats[n]) <= 1e-12


@pytest.mark.parametrize("case", ["large", "small"])
def test_svd_plan_matches_oracle(nd, case):
    rng = np.random.default_rng(91 if case == "large" else 92)
    dims = [(700, 600), (520, 560), (64, 90)] if case == "large" else [(40, 30), (25, 60), (7, 7)]
    A, mats = _matrix(rng, dims, decay=-6 if case == "large" else None)
    for kw in ({}, {"maxdim": 300 if case == "large" else 40, "cutoff": 1e-10}):
        plan = nd.SvdPlan(nd.BlockSparseTensor.from_oracle(A), **kw)
        plan.run(nd.BlockSparseTensor.from_oracle(A))
        _check(plan.result(), mats, kw)
        plan.destroy()


def test_svd_plan_graph_replay(nd):
    import torch
    rng = np.random.default_rng(93)
    dims = [(600, 500), (300, 320), (16, 16)]
    A, _ = _matrix(rng, dims)
    G = nd.BlockSparseTensor.from_oracle(A)
    kw = {"maxdim": 400, "cutoff": 1e-12}
    plan = nd.SvdPlan(G, **kw)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        plan.run(G)                                   # eager run outside the capture
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        plan.run(G)
    # new data in the same buffer, replayed
    A2, mats2 = _matrix(np.random.default_rng(94), dims)
    G.data.copy_(torch.from_numpy(A2.data).to(G.data.device))
    g.replay()
    torch.cuda.synchronize()
    res_graph = plan.result()
    got = (res_graph[0].data_numpy().copy(), [x.cpu().numpy().copy() for x in res_graph[1]],
           res_graph[2].data_numpy().copy(), res_graph[3].eigs.copy(), res_graph[3].truncerr, list(res_graph[4]))
    _check(res_graph, mats2, kw)
    plan.run(G)                                       # eager, same data
    res_eager = plan.result()
    np.testing.assert_array_equal(res_eager[0].data_numpy(), got[0])
    for a, b in zip(res_eager[1], got[1]):
        np.testing.assert_array_equal(a.cpu().numpy(), b)
    np.testing.assert_array_equal(res_eager[2].data_numpy(), got[2])
    np.testing.assert_array_equal(res_eager[3].eigs, got[3])
    assert res_eager[3].truncerr == got[4] and list(res_eager[4]) == got[5]
    plan.destroy()


def test_svd_plan_reports_noconv(nd):
    rng = np.random.default_rng(95)
    A, _ = _matrix(rng, [(50, 40), (30, 30)])
    h = nd.handle(0)
    h.call("nd_set_svd_max_sweeps", 0)
    try:
        plan = nd.SvdPlan(nd.BlockSparseTensor.from_oracle(A))
        plan.run(nd.BlockSparseTensor.from_oracle(A))
        assert plan.result() is None                  # the reference's svd returns nothing
        plan.destroy()
    finally:
        h.call("nd_set_svd_max_sweeps", -1)
