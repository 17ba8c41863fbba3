"""Dense contract! on the GPU vs the oracle (GPU).

Tolerances (relative Frobenius error vs the FP64 oracle):
  fp64   <= 1e-13   (the dense pair workload's bar)
  ozaki  <= 1e-10
  bf16x3 <= 1e-4
"""
import numpy as np
import pytest

from oracle import dense as odense
from oracle import networks

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-13, "ozaki": 1e-10, "bf16x3": 1e-4}


def _run(nd, a, la, b, lb, lr, precision, alpha=1.0, beta=0.0, r0=None):
    A = nd.DenseTensor.from_numpy(a)
    B = nd.DenseTensor.from_numpy(b)
    ref = odense.contract(a, la, b, lb, lr, alpha=alpha, beta=beta, r=None if r0 is None else r0.copy())
    R = nd.DenseTensor.from_numpy(r0 if r0 is not None else np.full(ref.shape, np.nan))
    nd.contract_(R, lr, A, la, B, lb, alpha, beta, precision)
    return R.to_numpy(), ref


@pytest.mark.parametrize("precision", ["fp64", "ozaki", "bf16x3"])
def test_dense_pair_workload(nd, precision):
    a, b = networks.dense_pair(seed=0)
    out, ref = _run(nd, a, (1, 2, -1), b, (-1, 3, 4), (1, 2, 3, 4), precision)
    assert odense.rel_frobenius_error(out, ref) <= TOL[precision]
    # followed by permutedims to (s, a, c, t)
    C = nd.DenseTensor.from_numpy(out)
    P = nd.permutedims(C, (2, 1, 4, 3))
    np.testing.assert_array_equal(P.to_numpy(), np.transpose(out, (1, 0, 3, 2)))


# a shape matrix in the spirit of test/base/test_contract.jl:7-264
SHAPES = [
    ((3, 4), (1, -1), (4, 5), (-1, 2), (1, 2)),
    ((3, 4), (-1, 1), (3, 5), (-1, 2), (2, 1)),
    ((4, 3), (-1, 1), (5, 4), (2, -1), (1, 2)),
    ((2, 3, 4), (1, -1, -2), (3, 4, 5), (-1, -2, 2), (1, 2)),
    ((2, 3, 4), (-2, 1, -1), (4, 5, 2), (-1, 2, -2), (2, 1)),
    ((6, 5, 4, 3), (1, -1, 2, -2), (3, 7, 5), (-2, 3, -1), (3, 2, 1)),
    ((5, 4), (1, 2), (3,), (3,), (2, 3, 1)),                      # outer product
    ((4, 5, 6), (-1, -2, -3), (6, 5, 4), (-3, -2, -1), ()),       # full contraction to a scalar
    ((130, 70), (1, -1), (70, 200), (-1, 2), (1, 2)),
    ((33, 65, 17), (1, -1, 2), (65, 19), (-1, 3), (3, 1, 2)),
    ((129, 600), (1, -1), (600, 65), (-1, 2), (1, 2)),           # K spans two exact chunks
]


@pytest.mark.parametrize("precision", ["fp64", "ozaki", "bf16x3"])
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: str(s[0]) + str(s[2]))
def test_shape_matrix(nd, shape, precision):
    da, la, db, lb, lr = shape
    rng = np.random.default_rng(abs(hash(shape)) % 2**32)
    a, b = rng.standard_normal(da), rng.standard_normal(db)
    out, ref = _run(nd, a, la, b, lb, lr, precision)
    assert odense.rel_frobenius_error(out, ref) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("alpha,beta", [(2.0, 0.0), (1.0, 1.0), (-0.5, 2.0), (0.0, 1.5)])
def test_alpha_beta(nd, precision, alpha, beta):
    rng = np.random.default_rng(5)
    a, b, r0 = rng.standard_normal((20, 30)), rng.standard_normal((30, 40)), rng.standard_normal((20, 40))
    out, ref = _run(nd, a, (1, -1), b, (-1, 2), (1, 2), precision, alpha, beta, r0)
    assert odense.rel_frobenius_error(out, ref) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("shape", [(4, 4, 4), (70, 90, 50)])
def test_gemm_alpha_beta_transpose_matrix(nd, precision, shape):
    """The reference's _gemm! matrix (NDTensors/test/test_dense.jl:216-235): alpha, beta in
    {0, 1, 2} and either operand transposed (expressed here by the label order), against
    numpy; 4 x 4 as in the reference and a larger rectangular case."""
    m, k, n = shape
    rng = np.random.default_rng(21)
    for alpha in (0.0, 1.0, 2.0):
        for beta in (0.0, 1.0, 2.0):
            for ta in "NT":
                for tb in "NT":
                    a = rng.standard_normal((m, k) if ta == "N" else (k, m))
                    b = rng.standard_normal((k, n) if tb == "N" else (n, k))
                    r0 = rng.standard_normal((m, n))
                    la = (1, -1) if ta == "N" else (-1, 1)
                    lb = (-1, 2) if tb == "N" else (2, -1)
                    out, _ = _run(nd, a, la, b, lb, (1, 2), precision, alpha, beta, r0)
                    opa = a if ta == "N" else a.T
                    opb = b if tb == "N" else b.T
                    expect = alpha * (opa @ opb) + beta * r0
                    if alpha == 0.0 and beta == 0.0:
                        assert not np.any(out), (ta, tb)          # R overwritten with zeros
                    else:
                        assert odense.rel_frobenius_error(out, expect) <= TOL[precision], (alpha, beta, ta, tb)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (-0.5, 2.0)])
def test_long_k_small_output(nd, precision, alpha, beta):
    """Tiny M x N with K = 3e5 (the W-cotangent shape of the H_eff gradient): the FP64
    path splits K across CTAs and sums the partial tiles in a fixed order."""
    rng = np.random.default_rng(21)
    a = rng.standard_normal((10, 600, 500))
    b = rng.standard_normal((500, 600, 12))
    r0 = rng.standard_normal((10, 12))
    out, ref = _run(nd, a, (1, -1, -2), b, (-2, -1, 2), (1, 2), precision, alpha, beta, r0)
    assert odense.rel_frobenius_error(out, ref) <= TOL[precision]
    out2, _ = _run(nd, a, (1, -1, -2), b, (-2, -1, 2), (1, 2), precision, alpha, beta, r0)
    np.testing.assert_array_equal(out, out2)          # deterministic reduction order


@pytest.mark.parametrize("lr", [(1, 2, 3), (2, 1, 3)])
def test_scalar_branch_overwrites_nan(nd, lr):
    # NDTensors/test/test_dense.jl:237-259
    rng = np.random.default_rng(6)
    t1 = rng.standard_normal((2, 2, 1))
    t2 = rng.standard_normal((1, 1))
    R = nd.DenseTensor.from_numpy(np.full((2, 2, 1), np.nan))
    nd.contract_(R, lr, nd.DenseTensor.from_numpy(t1), (1, 2, -1), nd.DenseTensor.from_numpy(t2), (-1, 1))
    ref = np.full((2, 2, 1), np.nan)
    odense.contract_into(ref, lr, t1, (1, 2, -1), t2, (-1, 1))
    assert not np.isnan(R.to_numpy()).any()
    np.testing.assert_allclose(R.to_numpy(), ref, rtol=1e-15)


def test_ozaki_adversarial_digits(nd):
    """Every leading digit at +-128 with aligned signs: each exact-level chunk sum
    reaches 2^24, the largest value the FP32 TMEM accumulator holds exactly."""
    rng = np.random.default_rng(7)
    K = 1024
    s = np.where(rng.random(K) < 0.5, -1.0, 1.0)
    x = 1.0 - 2.0 ** -10 + rng.random((128, K)) * 2.0 ** -12
    y = 1.0 - 2.0 ** -10 + rng.random((K, 64)) * 2.0 ** -12
    a = x * s[None, :]
    b = y * s[:, None]
    out, ref = _run(nd, a, (1, -1), b, (-1, 2), (1, 2), "ozaki")
    # 5 digits keep 39 bits relative to each row/column maximum
    assert odense.rel_frobenius_error(out, ref) <= 2.0 ** -36


@pytest.mark.parametrize("slices,tol", [(3, 1e-5), (4, 1e-8), (5, 1e-10), (6, 1e-10)])
def test_ozaki_slice_counts(nd, slices, tol):
    """Every slice count the library accepts (3..6): each lays its levels into the
    [L2 | L3 | T4 | T5+] accumulator slot with a different MMA schedule (N = 64 r
    runs per A slice, A-collector reuse for the products that share a slice)."""
    rng = np.random.default_rng(30 + slices)
    a, b = rng.standard_normal((300, 700)), rng.standard_normal((700, 200))
    h = nd.handle(0)
    h.call("nd_set_ozaki_slices", slices)
    try:
        out, ref = _run(nd, a, (1, -1), b, (-1, 2), (1, 2), "ozaki")
    finally:
        h.call("nd_set_ozaki_slices", 5)
    assert odense.rel_frobenius_error(out, ref) <= tol


def test_ozaki_wide_dynamic_range(nd):
    rng = np.random.default_rng(8)
    a = rng.standard_normal((200, 300)) * np.exp(rng.uniform(-20, 20, (200, 1)))
    b = rng.standard_normal((300, 100)) * np.exp(rng.uniform(-20, 20, (1, 100)))
    out, ref = _run(nd, a, (1, -1), b, (-1, 2), (1, 2), "ozaki")
    assert odense.rel_frobenius_error(out, ref) <= 1e-10


def test_bad_labels_rejected(nd):
    a = nd.DenseTensor.from_numpy(np.ones((2, 3)))
    b = nd.DenseTensor.from_numpy(np.ones((3, 4)))
    r = nd.DenseTensor.from_numpy(np.ones((2, 4)))
    with pytest.raises(nd.NDError):
        nd.contract_(r, (1, 5), a, (1, -1), b, (-1, 2))
    with pytest.raises(nd.NDError):
        nd.contract_(nd.DenseTensor.from_numpy(np.ones((2, 4))), (1, 2), a, (1, -1),
                     nd.DenseTensor.from_numpy(np.ones((4, 4))), (-1, 2))


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_dense_state_reuse_and_capture(nd, precision):
    """Repeated dense contractions of one shape reuse the cached device state: results
    are identical, other shapes interleave freely, and after one eager call the
    contraction can be captured into a CUDA graph and replayed."""
    import ctypes as C
    import torch
    rng = np.random.default_rng(31)
    a, b = rng.standard_normal((96, 3, 80)), rng.standard_normal((80, 3, 70))
    la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
    ref = odense.contract(a, la, b, lb, lr)
    A, B = nd.DenseTensor.from_numpy(a), nd.DenseTensor.from_numpy(b)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        R = nd.DenseTensor.empty(ref.shape)
        nd.contract_(R, lr, A, la, B, lb, precision=precision)
        first = R.to_numpy()
        assert odense.rel_frobenius_error(first, ref) <= TOL[precision]
        other, oref = _run(nd, a[:50], la, b, lb, lr, precision)           # a second shape in between
        assert odense.rel_frobenius_error(other, oref) <= TOL[precision]
        nd.contract_(R, lr, A, la, B, lb, precision=precision)
        np.testing.assert_array_equal(R.to_numpy(), first)
        h = nd.handle(0)
        R.data.zero_()
        torch.cuda.synchronize()
        h.call("nd_graph_begin")
        nd.contract_(R, lr, A, la, B, lb, precision=precision)
        ge = C.c_void_p()
        h.call("nd_graph_end", C.byref(ge))
        for _ in range(2):
            R.data.zero_()
            h.call("nd_graph_launch", ge)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(R.to_numpy(), first)
        h.lib.nd_graph_destroy(ge)
        # a shape never run eagerly cannot be built inside a capture
        R2 = nd.DenseTensor.empty((96, 3, 3, 71))
        B2 = nd.DenseTensor.from_numpy(rng.standard_normal((80, 3, 71)))
        h.call("nd_graph_begin")
        with pytest.raises(nd.NDError):
            nd.contract_(R2, lr, A, la, B2, lb, precision=precision)
        h.call("nd_graph_end", C.byref(ge))
        if ge.value:
            h.lib.nd_graph_destroy(ge)


@pytest.mark.parametrize("precision", ["ozaki", "bf16x3"])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (2.0, 0.0), (-0.5, 2.0)])
def test_skinny_split_precision_dynamic_range(nd, precision, alpha, beta):
    """Skinny pairs (N <= 8, K <= 32) in the split precisions run on the FP64 CUDA-core
    kernel: rows spanning 2^-300 .. 2^300, a B column of tiny values, zeros, and the
    alpha / beta store modes, held row by row to 1e-12."""
    rng = np.random.default_rng(40)
    a = rng.standard_normal((3000, 7, 3)) * 2.0 ** rng.integers(-300, 300, (3000, 1, 1))
    a[::17, 2, :] = 0.0
    b = rng.standard_normal((3, 7, 5))
    b[:, :, 4] *= 2.0 ** -200
    r0 = rng.standard_normal((3000, 5))
    out, ref = _run(nd, a, (1, -1, -2), b, (-2, -1, 2), (1, 2), precision, alpha, beta, r0)
    # per output row: the row scales differ by up to 2^600, so compare row by row
    num = np.linalg.norm(out - ref, axis=1)
    den = np.linalg.norm(ref, axis=1) + 1e-300
    assert np.max(num / den) <= 1e-12


@pytest.mark.parametrize("k", [4, 20])
def test_skinny_propagates_inf_nan(nd, k):
    """Inf and NaN operands of skinny pairs propagate as in FP64 BLAS."""
    a = np.ones((600, k))
    a[3, 1], a[7, 2] = np.nan, np.inf
    b = np.ones((k, 3))
    out, ref = _run(nd, a, (1, -1), b, (-1, 2), (1, 2), "ozaki")
    assert np.isnan(out[3]).all() and np.isinf(out[7]).all()
    mask = np.ones(600, bool)
    mask[[3, 7]] = False
    np.testing.assert_allclose(out[mask], ref[mask], rtol=1e-15)
