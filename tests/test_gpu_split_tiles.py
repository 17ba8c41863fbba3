"""Both output-tile shapes of the split-precision GEMM against the oracle (GPU).

Shape 0 (the default) runs 128 x 64 tiles on single CTAs; shape 1 runs 256 x 64 tiles on
pairs of CTAs (tcgen05.mma with M = 256, each CTA staging half of every B slice).
Each test runs under both: every slice count, row counts that leave the odd CTA of a
pair past the last row, N and K that are not multiples of the tile, K spanning several
exact 512-wide accumulation chunks, general alpha / beta, the 2^24 worst case of the
exact FP32 accumulation, and a grouped block-sparse contraction with several pairs per
output block.  Tolerances are the split precisions' bars (relative Frobenius error vs
the FP64 oracle): Ozaki 1e-10 at 5-6 slices, 1e-8 at 4, 1e-5 at 3; 3xBF16 1e-4.
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import dense as odense
from oracle import networks, qn

pytestmark = pytest.mark.gpu
SLICE_TOL = {3: 1e-5, 4: 1e-8, 5: 1e-10, 6: 1e-10}


@pytest.fixture(params=[1, 0], ids=["pair256x64", "single128x64"])
def tile(nd, request):
    h = nd.handle(0)
    h.call("nd_set_split_tile", request.param)
    yield request.param
    h.call("nd_set_split_tile", 0)


def _run(nd, a, la, b, lb, lr, precision, alpha=1.0, beta=0.0, r0=None):
    ref = odense.contract(a, la, b, lb, lr)
    if r0 is None:
        r0 = np.full(ref.shape, np.nan) if beta == 0.0 else np.zeros(ref.shape)
    want = alpha * ref + (beta * r0 if beta != 0.0 else 0.0)
    R = nd.DenseTensor.from_numpy(r0)
    nd.contract_(R, lr, nd.DenseTensor.from_numpy(a), la, nd.DenseTensor.from_numpy(b), lb, alpha, beta,
                 precision=precision)
    return R.to_numpy(), want


@pytest.mark.parametrize("slices", [3, 4, 5, 6])
@pytest.mark.parametrize("m,n,k", [(401, 70, 1300), (100, 64, 20), (256, 130, 513), (700, 33, 2049)])
def test_tiles_slice_counts_ragged(nd, tile, slices, m, n, k):
    rng = np.random.default_rng(1000 + m + n + k + slices)
    a, b = rng.standard_normal((m, k)), rng.standard_normal((k, n))
    h = nd.handle(0)
    h.call("nd_set_ozaki_slices", slices)
    try:
        out, ref = _run(nd, a, (1, -1), b, (-1, 2), (1, 2), "ozaki")
    finally:
        h.call("nd_set_ozaki_slices", 5)
    assert odense.rel_frobenius_error(out, ref) <= SLICE_TOL[slices]


@pytest.mark.parametrize("precision", ["ozaki", "bf16x3"])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (2.0, 0.0), (-0.5, 2.0)])
def test_tiles_alpha_beta_permuted(nd, tile, precision, alpha, beta):
    rng = np.random.default_rng(77)
    a, b = rng.standard_normal((30, 70, 45)), rng.standard_normal((45, 90, 30))
    r0 = rng.standard_normal((90, 70))
    out, ref = _run(nd, a, (-2, 1, -1), b, (-1, 2, -2), (2, 1), precision, alpha, beta, r0)
    assert odense.rel_frobenius_error(out, ref) <= (1e-10 if precision == "ozaki" else 1e-4)


def test_tiles_adversarial_digits(nd, tile):
    """Leading digits at +-128 with aligned signs: every exact chunk sum reaches 2^24."""
    rng = np.random.default_rng(7)
    K = 1024
    s = np.where(rng.random(K) < 0.5, -1.0, 1.0)
    a = (1.0 - 2.0 ** -10 + rng.random((300, K)) * 2.0 ** -12) * s[None, :]
    b = (1.0 - 2.0 ** -10 + rng.random((K, 64)) * 2.0 ** -12) * s[:, None]
    out, ref = _run(nd, a, (1, -1), b, (-1, 2), (1, 2), "ozaki")
    assert odense.rel_frobenius_error(out, ref) <= 2.0 ** -36


@pytest.mark.parametrize("precision", ["ozaki", "bf16x3"])
def test_tiles_grouped_blocksparse(nd, tile, precision):
    """Several block pairs accumulate into each output block (the Multithreading-doc
    structure) and the QN pair workload, through the grouped launch."""
    rng = np.random.default_rng(3)
    d = 24
    i1 = qn.QNIndex(((0, d), (1, d)), 1, "i1")
    i2 = qn.QNIndex(((0, d), (1, d)), 1, "i2")
    inds = [i1.primed(), i2.primed(), i1.dag(), i2.dag()]
    A = obs.random_blocksparse(rng, [x.dims for x in inds], qn.nzblocks(0, inds))
    B = obs.random_blocksparse(rng, [x.dims for x in inds], qn.nzblocks(0, inds))
    tol = 1e-10 if precision == "ozaki" else 1e-4
    P, Q, _ = networks.qn_pair(2048)
    for (T1, l1, T2, l2, lr) in ((A, (1, 2, -1, -2), B, (-1, -2, 3, 4), (1, 2, 3, 4)),
                                 (P, (1, 2, -1), Q, (-1, 3, 4), (1, 2, 3, 4))):
        ref, _ = obs.contract(T1, l1, T2, l2, lr)
        G1, G2 = nd.BlockSparseTensor.from_oracle(T1), nd.BlockSparseTensor.from_oracle(T2)
        R = nd.contract_blocksparse(G1, l1, G2, l2, lr, precision=precision, plan=nd.ContractionPlan(G1, l1, G2, l2, lr))
        assert odense.rel_frobenius_error(R.data_numpy(), ref.data) <= tol


def test_tiles_agree(nd):
    """The two tile shapes accumulate the same digit products into each level in the
    same order (slice p major, q minor) and drain the same chunks, so their Ozaki
    results agree to rounding of the FP32 tail levels (bar 1e-14)."""
    rng = np.random.default_rng(88)
    a, b = rng.standard_normal((517, 1500)), rng.standard_normal((1500, 200))
    h = nd.handle(0)
    outs = []
    try:
        for t in (1, 0):
            h.call("nd_set_split_tile", t)
            outs.append(_run(nd, a, (1, -1), b, (-1, 2), (1, 2), "ozaki")[0])
    finally:
        h.call("nd_set_split_tile", 0)
    assert odense.rel_frobenius_error(outs[0], outs[1]) <= 1e-14
