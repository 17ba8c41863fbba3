"""Device Lanczos (krylov.py) vs the oracle recurrence (GPU).

The same Krylov recurrence (full re-orthogonalisation, classical Gram-Schmidt twice)
run on the device, eagerly and captured in one CUDA graph, against the numpy
restatement in oracle/krylov.py: tridiagonal coefficients and the lowest Ritz value
agree to FP64 roundoff; the captured and eager runs agree bit for bit.
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import krylov as okr
from oracle import networks

pytestmark = pytest.mark.gpu


def test_lanczos_symmetric_dense_operator(nd):
    import torch
    rng = np.random.default_rng(51)
    n = 1536
    m = rng.standard_normal((n, n))
    H = (m + m.T) / np.sqrt(n)
    Hd = nd.DenseTensor.from_numpy(H)
    v0 = rng.standard_normal(n)

    def apply(x, out):
        X = nd.DenseTensor((n,), x)
        Y = nd.DenseTensor((n,), out)
        nd.contract_(Y, (1,), Hd, (1, -1), X, (-1,))
        return out

    ref_val, ref_vec, ref_a, ref_b = okr.lanczos(lambda x: H @ x, v0, 30)
    res = nd.lanczos(apply, torch.from_numpy(v0).cuda(), krylovdim=30)
    np.testing.assert_allclose(res.alpha, ref_a, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(res.beta, ref_b, rtol=1e-10, atol=1e-12)
    assert abs(res.value - ref_val) <= 1e-10 * abs(ref_val)
    x = res.vector.cpu().numpy()
    assert abs(abs(x @ ref_vec) - 1.0) <= 1e-8


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_lanczos_heff_graph_matches_eager_and_oracle(nd, precision):
    import torch
    net = networks.qn_heff(chi=256, seed=52)
    steps = networks.heff_steps()
    G = {k: nd.BlockSparseTensor.from_oracle(net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    op = nd.HeffOperator(G["L"], G["W1"], G["W2"], G["R"], G["psi"], steps, precision=precision)
    v0 = G["psi"].data.clone()
    eager = nd.Lanczos(op.apply, op.n, krylovdim=8).run(v0)
    lz = nd.Lanczos(op.apply, op.n, krylovdim=8, graph=True)
    first = lz.run(v0)
    second = lz.run(v0)                                   # replay of the captured graph
    np.testing.assert_array_equal(first.alpha, eager.alpha)
    np.testing.assert_array_equal(second.beta, eager.beta)
    assert first.value == eager.value

    psi = net["psi"]

    def apply_oracle(x):
        t = obs.BlockSparseTensor(psi.inds, psi.blocks, psi.offsets, x)
        y, _ = obs.contract(net["L"], steps[0][0], t, steps[0][1], steps[0][2])
        for (a, b, c), key in zip(steps[1:], ("W1", "W2", "R")):
            y, _ = obs.contract(y, a, net[key], b, c)
        out = np.empty_like(x)
        where = {tuple(b): o for b, o in zip(y.blocks, y.offsets)}
        for b, off in zip(psi.blocks, psi.offsets):
            nb = int(np.prod(psi.blockdims(b)))
            out[off:off + nb] = y.data[where[tuple(b)]:where[tuple(b)] + nb]
        return out

    ref_val, _, ref_a, ref_b = okr.lanczos(apply_oracle, psi.data.copy(), 8)
    tol = 1e-11 if precision == "fp64" else 1e-8
    np.testing.assert_allclose(eager.alpha, ref_a, rtol=tol, atol=tol * np.abs(ref_a).max())
    np.testing.assert_allclose(eager.beta, ref_b, rtol=tol, atol=tol * np.abs(ref_b).max())
    assert abs(eager.value - ref_val) <= tol * abs(ref_val)
