"""Autotuner: per block-size-histogram choice of execution parameters (GPU).

With tuning on, the first execution of a contraction times every candidate on
the real operands and caches the fastest under its histogram key; the result
must still match the oracle, the cache must survive a save / load round trip,
and a malformed cache file must be refused.
"""
import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import dense as odense
from oracle import networks

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-13, "ozaki": 1e-10}


@pytest.fixture
def tuned(nd):
    h = nd.handle(0)
    h.tune(True)
    yield h
    h.tune(False)


@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_tuned_contraction_matches_oracle(nd, tuned, precision, tmp_path):
    A, B, _ = networks.qn_pair(384, seed=41 if precision == "fp64" else 42)
    la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
    ref, _ = obs.contract(A, la, B, lb, lr)
    GA, GB = nd.BlockSparseTensor.from_oracle(A), nd.BlockSparseTensor.from_oracle(B)
    before = tuned.tune_count()
    plan = nd.ContractionPlan(GA, la, GB, lb, lr)
    R = nd.contract_blocksparse(GA, la, GB, lb, lr, precision=precision, plan=plan)
    assert odense.rel_frobenius_error(R.data_numpy(), ref.data) <= TOL[precision]
    assert tuned.tune_count() >= before + 1
    # repeated calls reuse the tuned state and stay correct
    R2 = nd.contract_blocksparse(GA, la, GB, lb, lr, precision=precision, plan=plan)
    np.testing.assert_array_equal(R2.data_numpy(), R.data_numpy())
    # a second plan of the same structure hits the cache (no new entry)
    n1 = tuned.tune_count()
    plan2 = nd.ContractionPlan(GA, la, GB, lb, lr)
    R3 = nd.contract_blocksparse(GA, la, GB, lb, lr, precision=precision, plan=plan2)
    assert tuned.tune_count() == n1
    np.testing.assert_array_equal(R3.data_numpy(), R.data_numpy())
    # save / load round trip into a fresh handle
    path = tmp_path / "tune.txt"
    tuned.tune_save(path)
    text = path.read_text().splitlines()
    assert text[0].startswith("#") and len(text) == n1 + 1
    from ndtensors_gb300._lib import Handle
    h2 = Handle(0)
    try:
        h2.tune_load(path)
        assert h2.tune_count() == n1
    finally:
        h2.close()


def test_tuned_adjoint(nd, tuned):
    """Both cotangents in one tuned grouped launch (two jobs)."""
    from oracle.adjoint import contract_pullback
    A, B, _ = networks.qn_pair(256, seed=43)
    la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
    R, _ = obs.contract(A, la, B, lb, lr)
    rng = np.random.default_rng(44)
    Rbar = obs.BlockSparseTensor(R.inds, R.blocks, R.offsets, rng.standard_normal(R.nnz))
    gA, gB = contract_pullback(A.to_dense(), (1, 2, 5), B.to_dense(), (5, 3, 4), (1, 2, 3, 4), Rbar.to_dense())
    GA, GB = nd.BlockSparseTensor.from_oracle(A), nd.BlockSparseTensor.from_oracle(B)
    before = tuned.tune_count()
    y, pullback = nd.contract_rrule(GA, la, GB, lb, lr)
    import torch
    abar, bbar = pullback(torch.from_numpy(Rbar.data).to(y.data.device))
    assert tuned.tune_count() >= before + 1
    Ab = obs.BlockSparseTensor(A.inds, A.blocks, A.offsets, abar.data_numpy()).to_dense()
    Bb = obs.BlockSparseTensor(B.inds, B.blocks, B.offsets, bbar.data_numpy()).to_dense()
    assert odense.rel_frobenius_error(Ab, gA) <= 1e-13
    assert odense.rel_frobenius_error(Bb, gB) <= 1e-13


def test_tune_load_rejects_malformed(nd, tmp_path):
    h = nd.handle(0)
    n = h.tune_count()
    bad = tmp_path / "bad.txt"
    bad.write_text("# header\nsm152/p0/s0/1.1.1x1\t4\tseven\t1.0\t1.0\n")
    with pytest.raises(nd.NDError):
        h.tune_load(bad)
    assert h.tune_count() == n
    with pytest.raises(nd.NDError):
        h.tune_load(tmp_path / "missing.txt")
