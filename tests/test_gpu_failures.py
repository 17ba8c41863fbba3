"""Failure paths that the library reports instead of hanging or aborting (GPU).

- A device-side wait that runs past the handle's spin limit makes the call report
  ND_ERR_TIMEOUT: the TMA pipeline of permutedims (nd_set_permute_path 1; mbarrier waits) and the grid
  barriers of the blockwise SVD.  The limit is set to one or two polls, far below the
  time a copy or a neighbouring CTA needs, so the waits run out; each kernel still
  waits for its own copies in flight before it exits.  The same handle then runs a
  normal call with the default limit and gets the right answer.
- An SVD that does not converge within the sweep limit: with the limit set to 0 the
  library returns ND_ERR_NOCONV and the Python mirror's ``svd`` returns None, as the
  reference's ``svd`` returns ``nothing`` (NDTensors/src/linearalgebra/linearalgebra.jl:120-127,
  NDTensors/src/blocksparse/linearalgebra.jl:65-67).
No GPU fault is involved: every access stays in bounds and every wait is bounded.
"""
import numpy as np
import pytest

from oracle import blocksparse as obs

pytestmark = pytest.mark.gpu
ND_ERR_NOCONV, ND_ERR_TIMEOUT = 3, 4


def _svd_input(seed=5):
    rng = np.random.default_rng(seed)
    mats = [rng.standard_normal((600, 500)), rng.standard_normal((90, 120))]
    inds = [[600, 90], [500, 120]]
    blocks = [(1, 1), (2, 2)]
    offs, _ = obs.blockoffsets(blocks, inds)
    return mats, obs.BlockSparseTensor(inds, blocks, offs, np.concatenate([m.reshape(-1, order="F") for m in mats]))


def test_permute_wait_timeout_then_recovers(nd):
    import torch
    dims, perm = (1024, 1024, 32), (2, 1, 3)            # 256 MiB, the TMA transpose path
    T = nd.DenseTensor(dims, torch.randn(int(np.prod(dims)), dtype=torch.float64, device="cuda"))
    R = nd.DenseTensor.empty(tuple(dims[p - 1] for p in perm))
    h = nd.handle(0)
    h.call("nd_set_permute_path", 1)
    try:
        try:
            h.call("nd_set_spin_limit", 1)
            with pytest.raises(nd.NDError) as e:
                nd.permutedims_(R, T, perm)
                h.sync()
            assert e.value.status == ND_ERR_TIMEOUT
        finally:
            h.call("nd_set_spin_limit", 0)
        nd.permutedims_(R, T, perm)
    finally:
        h.call("nd_set_permute_path", 0)
    h.sync()
    want = T.data.view(*reversed(dims)).permute(0, 2, 1)        # row-major view of the column-major perm
    assert torch.equal(R.data.view(*reversed(R.dims)), want.contiguous())


def test_svd_grid_barrier_timeout_then_recovers(nd):
    mats, A = _svd_input()
    GA = nd.BlockSparseTensor.from_oracle(A)
    h = nd.handle(0)
    try:
        h.call("nd_set_spin_limit", 1)
        with pytest.raises(nd.NDError) as e:
            nd.svd(GA)
        assert e.value.status == ND_ERR_TIMEOUT
    finally:
        h.call("nd_set_spin_limit", 0)
    U, S, V, spec, kept = nd.svd(GA)
    for n, m in enumerate(mats):
        np.testing.assert_allclose(S[n].cpu().numpy(), np.linalg.svd(m, compute_uv=False), rtol=0,
                                   atol=1e-12 * np.linalg.norm(m, 2))


def test_svd_noconvergence_returns_none(nd):
    import ctypes as C
    mats, A = _svd_input(6)
    GA = nd.BlockSparseTensor.from_oracle(A)
    h = nd.handle(0)
    try:
        h.call("nd_set_svd_max_sweeps", 0)
        assert nd.svd(GA) is None
        # the C ABI reports the status itself
        from ndtensors_gb300._lib import i64arr
        import torch
        rows, cols = [600, 90], [500, 120]
        U = torch.empty(600 * 500 + 90 * 90, dtype=torch.float64, device="cuda")
        S = torch.empty(590, dtype=torch.float64, device="cuda")
        V = torch.empty(500 * 500 + 120 * 90, dtype=torch.float64, device="cuda")
        kept = (C.c_int32 * 2)()
        spec = (C.c_double * 590)()
        sl, te, dc = C.c_int32(), C.c_double(), C.c_double()
        st = h.lib.nd_bs_svd_f64(h.ptr, 2, i64arr(rows), i64arr(cols), i64arr(GA.offsets), C.c_void_p(GA.data.data_ptr()),
                                 C.c_void_p(U.data_ptr()), C.c_void_p(S.data_ptr()), C.c_void_p(V.data_ptr()),
                                 1, -1, -1.0, 0, 1, 0, kept, spec, C.byref(sl), C.byref(te), C.byref(dc))
        assert st == ND_ERR_NOCONV
    finally:
        h.call("nd_set_svd_max_sweeps", -1)
    out = nd.svd(GA)
    assert out is not None
    for n, m in enumerate(mats):
        np.testing.assert_allclose(out[1][n].cpu().numpy(), np.linalg.svd(m, compute_uv=False), rtol=0,
                                   atol=1e-12 * np.linalg.norm(m, 2))
