"""The sweep-step operations around the contraction, in the library's own kernels (GPU).

- VectorInterface operations (ext/ITensorsVectorInterfaceExt/ITensorsVectorInterfaceExt.jl:5-84)
  through the C ABI: inner, norm, scale, add, and the Gram-Schmidt basis forms, vs numpy
  to FP64 roundoff; repeated reductions are bit-identical (fixed reduction order).
- BlockSparse x block-diagonal DiagBlockSparse (NDTensors/src/blocksparse/diagblocksparse.jl:601-696)
  in the cases the column scaling does not cover: D fully contracted (a trace over the
  diagonal) and D with two free indices (the result is diagonal in them), vs the oracle
  contraction with D expanded to dense blocks; structure bit-exact, values to 1e-14.
- A plan whose output blocks are written at caller-given offsets.
- The Lanczos iteration, blockwise eigen and the diagonal contraction launch only the
  library's kernels: the CUDA kernels torch's profiler records are all library kernels
  (memcpy / memset activity aside).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import blocksparse as obs
from oracle import dense as odense
from oracle import networks, qn

pytestmark = pytest.mark.gpu


def _ptr(t, off=0):
    return C.c_void_p(t.data_ptr() + 8 * off)


def test_vector_interface_ops(nd):
    import torch
    h = nd.handle(0)
    rng = np.random.default_rng(81)
    n, k = 1_000_003, 7
    Vh = rng.standard_normal((k, n))
    xh, yh = rng.standard_normal(n), rng.standard_normal(n)
    V = torch.from_numpy(Vh).cuda()
    x, y = torch.from_numpy(xh).cuda(), torch.from_numpy(yh).cuda()
    out = torch.empty(k, dtype=torch.float64, device="cuda")
    h.call("nd_vec_inner_f64", n, _ptr(x), _ptr(y), _ptr(out))
    assert abs(out[0].item() - xh @ yh) <= 1e-12 * np.linalg.norm(xh) * np.linalg.norm(yh)
    h.call("nd_vec_norm_f64", n, _ptr(x), _ptr(out))
    assert abs(out[0].item() - np.linalg.norm(xh)) <= 1e-14 * np.linalg.norm(xh)
    h.call("nd_vec_dots_f64", n, k, _ptr(V), n, _ptr(x), _ptr(out))
    ref = Vh @ xh
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=0, atol=1e-12 * np.linalg.norm(xh) * np.sqrt(n))
    first = out.cpu().numpy().copy()
    h.call("nd_vec_dots_f64", n, k, _ptr(V), n, _ptr(x), _ptr(out))
    np.testing.assert_array_equal(out.cpu().numpy(), first)              # same reduction order every call
    w = y.clone()
    h.call("nd_vec_update_f64", n, k, _ptr(V), n, _ptr(out), -1.0, _ptr(w))
    np.testing.assert_allclose(w.cpu().numpy(), yh - Vh.T @ first, rtol=0, atol=1e-12 * np.abs(Vh.T @ first).max())
    s = torch.tensor([4.0], dtype=torch.float64, device="cuda")
    z = torch.empty_like(x)
    h.call("nd_vec_scale_f64", n, _ptr(x), _ptr(z), 2.0, _ptr(s), 1)     # z = 2 x / 4
    np.testing.assert_array_equal(z.cpu().numpy(), 2.0 * xh / 4.0)
    z.fill_(float("nan"))
    h.call("nd_vec_add_f64", n, _ptr(x), _ptr(z), 3.0, 0.0)              # beta = 0 overwrites NaN
    np.testing.assert_array_equal(z.cpu().numpy(), 3.0 * xh)
    h.call("nd_vec_add_f64", n, _ptr(y), _ptr(z), -1.0, 0.5)
    np.testing.assert_allclose(z.cpu().numpy(), 0.5 * 3.0 * xh - yh, rtol=1e-15, atol=1e-15)
    with pytest.raises(nd.NDError):
        h.call("nd_vec_dots_f64", n, 33, _ptr(V), n, _ptr(x), _ptr(out))   # more than 32 basis vectors


def _diag_case(nd, rng, T_inds, T_blocks, D_dims, D_blocks, lT, lD, lR):
    import torch
    T = obs.random_blocksparse(rng, T_inds, T_blocks)
    diags = [rng.standard_normal(min(D_dims[k][b[k] - 1] for k in range(len(b)))) for b in D_blocks]
    Dt = nd.DiagBlockSparseTensor.from_diagonals(D_dims, D_blocks, [torch.from_numpy(d).cuda() for d in diags])
    Dd = Dt.dense()
    Do = obs.BlockSparseTensor([list(i) for i in Dd.inds], Dd.blocks, Dd.offsets, Dd.data_numpy())
    # the dense expansion itself: the diagonal at (i, ..., i) and zeros elsewhere
    for b, dv in zip(D_blocks, diags):
        blk = Do.blockview(Do.blocks.index(tuple(b)))
        idx = np.arange(len(dv))
        np.testing.assert_array_equal(blk[(idx,) * len(b)], dv)
        assert np.count_nonzero(blk) <= len(dv)
    ref, _ = obs.contract(T, lT, Do, lD, lR)
    R = nd.contract(nd.BlockSparseTensor.from_oracle(T), lT, Dt, lD, lR)
    assert R.blocks == [tuple(b) for b in ref.blocks] and R.offsets == list(ref.offsets)
    if ref.nnz:
        assert odense.rel_frobenius_error(R.data_numpy(), ref.data) <= 1e-14
    return R


def test_diag_fully_contracted(nd):
    """R(a) = sum_i d_i T(a, i, i): D's two indices both contracted, several T blocks per output block."""
    rng = np.random.default_rng(82)
    inds = [[30, 40], [5, 7, 6], [5, 7, 6]]
    T_blocks = [(1, 1, 1), (1, 2, 2), (2, 3, 3), (2, 1, 1), (1, 3, 3), (2, 2, 1)]
    D_dims = [(5, 7, 6), (5, 7, 6)]
    _diag_case(nd, rng, inds, T_blocks, D_dims, [(1, 1), (2, 2), (3, 3)], (1, -1, -2), (-1, -2), (1,))


def test_diag_two_free_indices(nd):
    """D of order 3 with one contracted and two free indices: R(x, i, i) = d_i T(x, i), zero off the diagonal."""
    rng = np.random.default_rng(83)
    inds = [[9, 11], [4, 6]]
    T_blocks = [(1, 1), (2, 2), (1, 2)]
    D_dims = [(4, 6), (4, 6), (4, 6)]
    _diag_case(nd, rng, inds, T_blocks, D_dims, [(1, 1, 1), (2, 2, 2)], (1, -1), (-1, 2, 3), (1, 2, 3))


def test_diag_rectangular_blocks(nd):
    """Non-square diagonal blocks (diagonal length min(dims)): the columns past it are zero."""
    rng = np.random.default_rng(84)
    inds = [[13, 8], [5, 9]]
    _diag_case(nd, rng, inds, [(1, 1), (2, 2), (2, 1)], [(5, 9), (7, 4)], [(1, 1), (2, 2)], (1, -1), (-1, 2), (1, 2))


def test_plan_output_offsets(nd):
    A, B, _ = networks.qn_pair(256, seed=85)
    la, lb, lr = (1, 2, -1), (-1, 3, 4), (1, 2, 3, 4)
    ref, _ = obs.contract(A, la, B, lb, lr)
    GA, GB = nd.BlockSparseTensor.from_oracle(A), nd.BlockSparseTensor.from_oracle(B)
    for prec in ("fp64", "ozaki"):
        p = nd.ContractionPlan(GA, la, GB, lb, lr)
        # reversed block order: block g written where the reference puts the last blocks
        sizes = [int(np.prod(ref.blockdims(b))) for b in ref.blocks]
        offs, o = [0] * len(sizes), 0
        for g in reversed(range(len(sizes))):
            offs[g] = o
            o += sizes[g]
        p.set_output_offsets(offs)
        R = nd.contract_blocksparse(GA, la, GB, lb, lr, precision=prec, plan=p)
        data = R.data_numpy()
        got = np.concatenate([data[offs[g]:offs[g] + sizes[g]] for g in range(len(sizes))])
        assert odense.rel_frobenius_error(got, ref.data) <= (1e-13 if prec == "fp64" else 1e-10)
        p.destroy()


def _library_kernels_only(fn):
    import torch
    from torch.profiler import ProfilerActivity, profile
    torch.cuda.synchronize()
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        fn()
        torch.cuda.synchronize()
    names = set()
    for ev in prof.events():
        if ev.device_type == torch.autograd.DeviceType.CUDA:
            names.add(ev.name)
    kernels = {n for n in names if not n.lower().startswith(("memcpy", "memset"))}
    if not kernels:
        pytest.skip("torch profiler recorded no CUDA kernels on this box")
    foreign = {n for n in kernels if any(t in n for t in ("at::", "at_cuda", "cublas", "gemv", "gemm_kernel", "cutlass",
                                                          "elementwise", "reduce_kernel", "index_", "Memset"))}
    assert not foreign, f"non-library kernels launched: {sorted(foreign)[:6]}"
    return kernels


def test_sweep_operations_launch_only_library_kernels(nd):
    import torch
    net = networks.qn_heff(chi=256, seed=86)
    steps = networks.heff_steps()
    G = {k: nd.BlockSparseTensor.from_oracle(net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    op = nd.HeffOperator(G["L"], G["W1"], G["W2"], G["R"], G["psi"], steps, precision="ozaki")
    lz = nd.Lanczos(op.apply, op.n, krylovdim=6)
    v0 = G["psi"].data.clone()
    lz.run(v0)                                            # plans and state built outside the profile
    k1 = _library_kernels_only(lambda: lz.run(v0))
    assert any("vec_dots" in n for n in k1) and any("split_gemm" in n for n in k1)
    # blockwise eigen and the diagonal contraction
    rng = np.random.default_rng(87)
    mats = [(lambda m: m + m.T)(rng.standard_normal((d, d))) for d in (30, 50)]
    offs, o = [], 0
    for m in mats:
        offs.append(o)
        o += m.size
    A = obs.BlockSparseTensor([[30, 50], [30, 50]], [(1, 1), (2, 2)], offs,
                              np.concatenate([m.reshape(-1, order="F") for m in mats]))
    GA = nd.BlockSparseTensor.from_oracle(A)
    nd.eigen(GA, maxdim=60)
    k2 = _library_kernels_only(lambda: nd.eigen(GA, maxdim=60))
    assert any("eig_finish" in n for n in k2)
    U, S, V, spec, kept = nd.svd(GA)
    Dt = nd.DiagBlockSparseTensor.from_diagonals([U.inds[1], U.inds[1]], [(i + 1, i + 1) for i in range(len(S))], S)
    nd.contract(U, (1, -1), Dt, (-1, 2))
    k3 = _library_kernels_only(lambda: nd.contract(U, (1, -1), Dt, (-1, 2)))
    assert any("bs_diag_contract" in n for n in k3)
