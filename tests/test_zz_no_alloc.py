"""The allocation-free Ozaki dense contraction (GPU).

nd_contract_dense_ozaki_noalloc_f64 serves callers that cannot allocate device
memory during a contraction (memory owned by another allocator with a hard
budget, or no tolerance for cudaMalloc's synchronisation).  It runs in a fixed
library-owned scratch array; this test checks, through the C ABI, that two
calls in a row give the same results as the regular entry point with
ND_PREC_OZAKI (tolerance 1e-10 relative Frobenius, the split-precision bar),
that stale scratch from the first call does not leak into the second, and that
a contraction larger than the scratch is refused with ND_ERR_ARG.  The file is
named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import dense as odense

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _call(nd, name, R, lr, A, la, B, lb, alpha=1.0, beta=0.0, precision=None):
    from ndtensors_gb300._lib import handle, i32arr, i64arr
    h = handle(0)
    args = [C.c_void_p(R.ptr()), len(R.dims), i64arr(R.dims), i32arr(lr),
            C.c_void_p(A.ptr()), len(A.dims), i64arr(A.dims), i32arr(la),
            C.c_void_p(B.ptr()), len(B.dims), i64arr(B.dims), i32arr(lb), float(alpha), float(beta)]
    if precision is not None:
        args.append(precision)
    return getattr(h.lib, name)(h.ptr, *args), h


def _case(nd, seed, da, la, db, lb, lr, alpha=1.0, beta=0.0):
    rng = np.random.default_rng(seed)
    a, b = rng.standard_normal(da), rng.standard_normal(db)
    ref = odense.contract(a, la, b, lb, lr)
    r0 = rng.standard_normal(ref.shape)
    A, B = nd.DenseTensor.from_numpy(a), nd.DenseTensor.from_numpy(b)
    R_new = nd.DenseTensor.from_numpy(r0)
    R_old = nd.DenseTensor.from_numpy(r0)
    st, h = _call(nd, "nd_contract_dense_ozaki_noalloc_f64", R_new, lr, A, la, B, lb, alpha, beta)
    assert st == 0, h.lib.nd_last_error(h.ptr)
    st, h = _call(nd, "nd_contract_dense_f64", R_old, lr, A, la, B, lb, alpha, beta, precision=1)
    assert st == 0, h.lib.nd_last_error(h.ptr)
    expect = alpha * ref + beta * r0
    out_new, out_old = R_new.to_numpy(), R_old.to_numpy()
    assert odense.rel_frobenius_error(out_new, out_old) <= TOL
    assert odense.rel_frobenius_error(out_new, expect) <= TOL


def test_noalloc_two_calls_match_regular_entry_point(nd):
    # first call: a large contraction fills much of the scratch
    _case(nd, 1, (384, 3, 200), (1, 2, -1), (200, 5, 100), (-1, 3, 4), (1, 2, 3, 4))
    # second call: a smaller, permuted contraction with alpha/beta reuses stale scratch
    _case(nd, 2, (40, 70, 30), (-2, 1, -1), (30, 90, 40), (-1, 2, -2), (2, 1), alpha=0.5, beta=-1.5)


def test_noalloc_rejects_oversize(nd):
    A = nd.DenseTensor.from_numpy(np.zeros((2048, 2048)))
    B = nd.DenseTensor.from_numpy(np.zeros((2048, 64)))
    R = nd.DenseTensor.from_numpy(np.zeros((2048, 64)))
    st, h = _call(nd, "nd_contract_dense_ozaki_noalloc_f64", R, (1, 2), A, (1, -1), B, (-1, 2))
    assert st == 1                                     # ND_ERR_ARG
    assert b"scratch" in h.lib.nd_last_error(h.ptr)
