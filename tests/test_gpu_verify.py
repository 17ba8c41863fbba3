"""Verify mode (nd_set_verify) on the GPU.

With verify mode on, a contraction in a split precision is computed a second time with
the FP64 kernels and the relative Frobenius distance of the two results is recorded.
These tests check that the recorded figure is the split result's actual error: it must
agree with the error measured against the oracle (within 2 % of it plus 1e-14, the
FP64 path's own distance from the oracle), that it stays under the precision's bar
(ozaki 1e-10, bf16x3 1e-4), that FP64 calls record 0, and that the call's own result
is unchanged by verification (bit-identical to the same call with the mode off).
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import dense as odense
from oracle import networks
from oracle.adjoint import contract_pullback

pytestmark = pytest.mark.gpu
TOL = {"ozaki": 1e-10, "bf16x3": 1e-4}


@pytest.fixture
def vh(nd):
    from ndtensors_gb300._lib import handle
    h = handle(0)
    h.verify(True)
    assert h.verify_last() == -1.0
    yield h
    h.verify(False)


def _agree(v, err, precision):
    assert 0.0 < v <= TOL[precision], (precision, v)
    assert abs(v - err) <= 0.02 * err + 1e-14, (precision, v, err)


@pytest.mark.parametrize("precision", ["ozaki", "bf16x3"])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (0.5, -1.5)])
def test_verify_dense(nd, vh, precision, alpha, beta):
    rng = np.random.default_rng(7)
    a, b = rng.standard_normal((96, 3, 200)), rng.standard_normal((200, 5, 80))
    la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
    ref = odense.contract(a, la, b, lb, lr)
    r0 = rng.standard_normal(ref.shape)
    expect = alpha * ref + beta * r0
    outs = []
    for on in (True, False):
        vh.verify(on)
        R = nd.DenseTensor.from_numpy(r0)
        nd.contract_(R, lr, nd.DenseTensor.from_numpy(a), la, nd.DenseTensor.from_numpy(b), lb,
                     alpha, beta, precision)
        outs.append(R.to_numpy())
        if on:
            _agree(vh.verify_last(), odense.rel_frobenius_error(outs[0], expect), precision)
    np.testing.assert_array_equal(outs[0], outs[1])
    vh.verify(True)
    R = nd.DenseTensor.from_numpy(r0)
    nd.contract_(R, lr, nd.DenseTensor.from_numpy(a), la, nd.DenseTensor.from_numpy(b), lb, alpha, beta, "fp64")
    assert vh.verify_last() == 0.0


@pytest.mark.parametrize("precision", ["ozaki", "bf16x3"])
def test_verify_blocksparse(nd, vh, precision):
    A, B, _ = networks.qn_pair(1024, seed=5)
    la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
    ref, _ = obs.contract(A, la, B, lb, lr)
    GA, GB = nd.BlockSparseTensor.from_oracle(A), nd.BlockSparseTensor.from_oracle(B)
    out = nd.contract(GA, la, GB, lb, lr, precision=precision).data_numpy()
    _agree(vh.verify_last(), odense.rel_frobenius_error(out, ref.data), precision)
    nd.contract(GA, la, GB, lb, lr, precision="fp64")
    assert vh.verify_last() == 0.0


def test_verify_adjoint(nd, vh):
    import torch
    A, B, _ = networks.qn_pair(512, seed=41)
    la, lb = (1, 2, -1), (-1, 3, 4)
    y, pb = nd.contract_rrule(nd.BlockSparseTensor.from_oracle(A), la, nd.BlockSparseTensor.from_oracle(B), lb,
                              precision="ozaki")
    R, _ = obs.contract(A, la, B, lb)
    ybar = torch.from_numpy(np.random.default_rng(42).standard_normal(R.nnz)).cuda()
    Ab, Bb = pb(ybar)
    v = vh.verify_last()
    gA, gB = contract_pullback(A.to_dense(), (1, 2, 5), B.to_dense(), (5, 3, 4), (1, 2, 3, 4),
                               obs.BlockSparseTensor(R.inds, R.blocks, R.offsets, ybar.cpu().numpy()).to_dense())
    Ad = obs.BlockSparseTensor(A.inds, A.blocks, A.offsets, Ab.data_numpy()).to_dense()
    Bd = obs.BlockSparseTensor(B.inds, B.blocks, B.offsets, Bb.data_numpy()).to_dense()
    # the recorded figure covers both cotangents together
    num = np.sum((Ad - gA) ** 2) + np.sum((Bd - gB) ** 2)
    den = np.sum(gA ** 2) + np.sum(gB ** 2)
    _agree(v, float(np.sqrt(num / den)), "ozaki")
