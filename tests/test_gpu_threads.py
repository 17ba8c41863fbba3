"""Concurrent handles on host threads give the serial results (GPU).

The reference runs the block pairs of a contraction on Julia tasks and tests that the
threaded result equals the serial one (test/threading/test_threading.jl:30-78).  Here the
equivalent contract is the C ABI's: a handle is driven by one host thread on its own
stream, and distinct handles are independent.  Four threads, each with its own handle
and CUDA stream, build block plans (host and device planner), run block-sparse
contractions in FP64 and Ozaki, a dense contraction and a permute, three times over,
concurrently; every result must equal, bit for bit, the same calls made serially on one
handle first.
"""
import ctypes as C
import threading

import numpy as np
import pytest

from oracle import networks

pytestmark = pytest.mark.gpu


def _work(nd, h, stream, GA, GB, a, b, placement):
    """One round of calls through handle h on stream; returns the results (numpy)."""
    import torch
    from ndtensors_gb300._lib import i32arr, i64arr
    out = []
    with torch.cuda.stream(stream):
        h.use_stream(stream.cuda_stream)
        h.call("nd_set_plan_placement", placement)
        la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
        d1, d2 = GA.desc(), GB.desc()
        plan = C.c_void_p()
        h.call("nd_bs_plan_create", C.byref(d1), i32arr(la), C.byref(d2), i32arr(lb), len(lr), i32arr(lr),
               C.byref(plan))
        try:
            npairs, nR, nnz = C.c_int32(), C.c_int32(), C.c_int64()
            h._check(h.lib.nd_bs_plan_sizes(plan, C.byref(npairs), C.byref(nR), C.byref(nnz)))
            for prec in (0, 1):
                R = torch.empty(nnz.value, dtype=torch.float64, device="cuda")
                h.call("nd_bs_contract_f64", plan, C.c_void_p(R.data_ptr()), C.c_void_p(GA.data.data_ptr()),
                       C.c_void_p(GB.data.data_ptr()), 1.0, prec)
                out.append(R)
        finally:
            h.lib.nd_bs_plan_destroy(plan)
        A, B = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
        Rd = torch.empty((a.shape[0], a.shape[1], b.shape[1], b.shape[2]), dtype=torch.float64, device="cuda")
        dims = lambda t: i64arr(tuple(t.shape)[::-1])          # column-major dims of a C-order array
        # column-major labels: A(i, s, k) B(k, t, j) -> R(i, s, t, j), written reversed for C order
        h.call("nd_contract_dense_f64", C.c_void_p(Rd.data_ptr()), 4, dims(Rd), i32arr((4, 3, 2, 1)),
               C.c_void_p(A.data_ptr()), 3, dims(A), i32arr((-1, 2, 1)),
               C.c_void_p(B.data_ptr()), 3, dims(B), i32arr((4, 3, -1)), 1.0, 0.0, 1)
        out.append(Rd)
        P = torch.empty_like(Rd)
        h.call("nd_permutedims_f64", C.c_void_p(P.data_ptr()), C.c_void_p(Rd.data_ptr()), 4, dims(Rd),
               i32arr((3, 1, 4, 2)), 1.0, 0.0)             # 1-based permutation
        out.append(P)
        stream.synchronize()
    return [t.cpu().numpy() for t in out]


def test_threads_match_serial(nd):
    import torch
    from ndtensors_gb300._lib import Handle
    A, B, _ = networks.qn_pair(1024, seed=11)
    GA, GB = nd.BlockSparseTensor.from_oracle(A), nd.BlockSparseTensor.from_oracle(B)
    rng = np.random.default_rng(12)
    a, b = rng.standard_normal((60, 3, 300)), rng.standard_normal((300, 4, 70))
    torch.cuda.synchronize()
    h0 = Handle(0)
    serial = _work(nd, h0, torch.cuda.Stream(), GA, GB, a, b, 0)
    h0.close()

    nthreads, rounds = 4, 3
    handles = [Handle(0) for _ in range(nthreads)]
    results, errors = {}, []
    barrier = threading.Barrier(nthreads)

    def run(t):
        try:
            s = torch.cuda.Stream()
            barrier.wait()
            results[t] = [_work(nd, handles[t], s, GA, GB, a, b, 1 if t % 2 else 2) for _ in range(rounds)]
        except Exception as e:                        # reported after the join
            errors.append((t, repr(e)))

    threads = [threading.Thread(target=run, args=(t,)) for t in range(nthreads)]
    for th in threads:
        th.start()
    for th in threads:
        th.join(timeout=600)
    for h in handles:
        h.close()
    assert not errors, errors
    assert len(results) == nthreads
    for t in range(nthreads):
        for r in range(rounds):
            for got, want in zip(results[t][r], serial):
                np.testing.assert_array_equal(got, want)
