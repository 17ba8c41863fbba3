"""permutedims kernel vs the oracle: bit-exact for plain copies (GPU)."""
import itertools

import numpy as np
import pytest

from oracle import dense as odense

pytestmark = pytest.mark.gpu

CASES = [
    ((256, 2, 2, 128), (2, 1, 4, 3)),       # the dense pair workload's output permute (a,s,t,c)->(s,a,c,t)
    ((7,), (1,)),
    ((5, 3), (2, 1)),
    ((64, 33), (2, 1)),
    ((2, 3, 4), (3, 1, 2)),
    ((31, 17, 9), (2, 3, 1)),
    ((16, 1, 8, 1, 4), (5, 3, 1, 4, 2)),
    ((6, 5, 4, 3, 2), (5, 4, 3, 2, 1)),
    ((3, 4, 5, 6, 2, 3), (2, 1, 6, 4, 3, 5)),
    ((2, 2, 2, 2, 2, 2, 2, 2), (8, 1, 7, 2, 6, 3, 5, 4)),
    ((130, 66, 3), (1, 3, 2)),
    ((4, 1, 1), (2, 3, 1)),
    # small extents: tiles over dimension groups (i over T's leading dims, j over R's)
    ((4, 8, 4, 8, 4, 8), (6, 5, 4, 3, 2, 1)),
    ((4, 8, 4, 8, 4, 8), (2, 1, 4, 3, 6, 5)),
    ((32, 8, 32, 8, 32), (5, 4, 3, 2, 1)),
    ((16, 8, 16, 8, 16), (3, 5, 1, 4, 2)),
    ((3, 5, 7, 11), (4, 2, 3, 1)),
    ((2, 3, 4, 5, 6, 7), (5, 6, 1, 2, 3, 4)),
]


@pytest.mark.parametrize("path", [0, 1])
@pytest.mark.parametrize("dims,perm", CASES)
def test_permutedims_exact(nd, dims, perm, path):
    """Both transposing paths (0: dimension-group tiles, 1: TMA tiles where they apply)."""
    rng = np.random.default_rng(hash((dims, perm)) % 2**32)
    a = rng.standard_normal(dims)
    T = nd.DenseTensor.from_numpy(a)
    h = nd.handle(0)
    h.call("nd_set_permute_path", path)
    try:
        R = nd.permutedims(T, perm)
    finally:
        h.call("nd_set_permute_path", 0)
    ref = odense.permutedims(a, perm)
    np.testing.assert_array_equal(R.to_numpy(), ref)


@pytest.mark.parametrize("alpha,beta", [(2.0, 0.0), (1.0, 1.0), (0.5, -1.5), (0.0, 2.0), (0.0, 0.0)])
def test_permutedims_alpha_beta(nd, alpha, beta):
    rng = np.random.default_rng(1)
    a = rng.standard_normal((40, 24, 3))
    r0 = rng.standard_normal((3, 40, 24))
    T = nd.DenseTensor.from_numpy(a)
    R = nd.DenseTensor.from_numpy(r0)
    nd.permutedims_(R, T, (3, 1, 2), alpha, beta)
    ref = odense.permutedims_into(r0.copy(), a, (3, 1, 2), alpha, beta)
    np.testing.assert_allclose(R.to_numpy(), ref, rtol=1e-15, atol=1e-15)


def test_permutedims_beta0_overwrites_nan(nd):
    a = np.random.default_rng(2).standard_normal((9, 70))
    T = nd.DenseTensor.from_numpy(a)
    R = nd.DenseTensor.from_numpy(np.full((70, 9), np.nan))
    nd.permutedims_(R, T, (2, 1), 1.0, 0.0)
    np.testing.assert_array_equal(R.to_numpy(), a.T)


def test_permutedims_large_exact(nd):
    # larger than L2 (129 MB): 3-D transpose of 24 M doubles (192 MB)
    import torch
    dims = (512, 96, 512)
    g = torch.Generator(device="cuda").manual_seed(3)
    data = torch.randn(int(np.prod(dims)), dtype=torch.float64, device="cuda", generator=g)
    T = nd.DenseTensor(dims, data)
    R = nd.permutedims(T, (3, 1, 2))
    a = data.cpu().numpy().reshape(dims, order="F")
    np.testing.assert_array_equal(R.to_numpy(), odense.permutedims(a, (3, 1, 2)))


def test_permutedims_small_extents_large_exact(nd):
    # larger than L2 (134 MB), every extent <= 64: the dimension-group tiling, rank-5 reversal
    import torch
    dims = (16, 32, 16, 32, 64)
    g = torch.Generator(device="cuda").manual_seed(4)
    data = torch.randn(int(np.prod(dims)), dtype=torch.float64, device="cuda", generator=g)
    T = nd.DenseTensor(dims, data)
    for perm in ((5, 4, 3, 2, 1), (2, 4, 1, 5, 3)):
        R = nd.permutedims(T, perm)
        a = data.cpu().numpy().reshape(dims, order="F")
        np.testing.assert_array_equal(R.to_numpy(), odense.permutedims(a, perm))


def test_bad_perm_rejected(nd):
    T = nd.DenseTensor.from_numpy(np.zeros((2, 3)))
    R = nd.DenseTensor.from_numpy(np.zeros((3, 2)))
    with pytest.raises(nd.NDError):
        import ctypes as C
        from ndtensors_gb300._lib import handle, i32arr, i64arr
        handle(0).call("nd_permutedims_f64", C.c_void_p(R.ptr()), C.c_void_p(T.ptr()), 2, i64arr((2, 3)),
                       i32arr((1, 1)), 1.0, 0.0)
