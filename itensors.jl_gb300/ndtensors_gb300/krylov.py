"""Lanczos eigensolver for an effective Hamiltonian, on the device.

A DMRG sweep solves its local eigenproblem with KrylovKit over the vector-space
interface the reference provides for ITensors
(ext/ITensorsVectorInterfaceExt/ITensorsVectorInterfaceExt.jl:5-84: add / add! /
inner / scale / scale!).  Here a vector is the flat FP64 data of a tensor with a
fixed block structure, and every VectorInterface operation is a library call
(nd_vec_inner_f64, nd_vec_norm_f64, nd_vec_scale_f64, nd_vec_add_f64, and the
basis forms nd_vec_dots_f64 / nd_vec_update_f64 for Gram-Schmidt).  The operator
is a sequence of library contractions (`HeffOperator`: the two-site H_eff applied
as L * psi, * W1, * W2, * R with cached plans and preallocated intermediates; the
last contraction writes straight into psi's block layout).

`lanczos` builds a Krylov basis of `krylovdim` vectors with full
re-orthogonalisation (classical Gram-Schmidt, twice).  Scalars (norms, alpha,
beta) stay on the device, so with ``graph=True`` the whole basis construction --
every matvec and every orthogonalisation -- is captured once into one CUDA graph
and replayed; the krylovdim x krylovdim tridiagonal problem is then solved on the
host.  No torch or cuBLAS kernel runs inside the loop.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import handle
from .contract import ContractionPlan, contract_blocksparse, get_plan
from .tensors import BlockSparseTensor


def _h(x):
    return handle(x.device.index or 0)


def _p(t, offset=0):
    return C.c_void_p(t.data_ptr() + 8 * offset)


def inner(x, y, out=None):
    """VectorInterface.inner(x, y) on flat real data: a device scalar (1-element tensor)."""
    import torch
    out = torch.empty(1, dtype=torch.float64, device=x.device) if out is None else out
    _h(x).call("nd_vec_inner_f64", int(x.numel()), _p(x), _p(y), _p(out))
    return out


def norm(x, out=None):
    """norm(x): a device scalar."""
    import torch
    out = torch.empty(1, dtype=torch.float64, device=x.device) if out is None else out
    _h(x).call("nd_vec_norm_f64", int(x.numel()), _p(x), _p(out))
    return out


def scale_(x, a):
    """VectorInterface.scale!(x, a): x *= a (a a number or a device scalar)."""
    return scale(x, a, out=x)


def scale(x, a, out=None, invert=False):
    """VectorInterface.scale(x, a): a * x (or x / a with invert), into `out`."""
    import torch
    out = torch.empty_like(x) if out is None else out
    if isinstance(a, torch.Tensor):
        _h(x).call("nd_vec_scale_f64", int(x.numel()), _p(x), _p(out), 1.0, _p(a), 1 if invert else 0)
    else:
        a = float(a)
        _h(x).call("nd_vec_scale_f64", int(x.numel()), _p(x), _p(out), 1.0 / a if invert else a, None, 0)
    return out


def add_(y, x, a=1.0, b=1.0):
    """VectorInterface.add!(y, x, a, b): y = b y + a x."""
    _h(x).call("nd_vec_add_f64", int(x.numel()), _p(x), _p(y), float(a), float(b))
    return y


class HeffOperator:
    """x -> H_eff x for the two-site network (L, W1, W2, R) on a fixed psi structure.

    Plans and the intermediates are built once.  The last contraction's plan is the
    operator's own (not the shared plan cache) and writes each output block at psi's
    offset for that block, so the operator maps the vector space onto itself with no
    gather and can be captured.
    """

    def __init__(self, L, W1, W2, R, psi: BlockSparseTensor, steps, precision="ozaki"):
        import torch
        self.steps, self.precision = steps, precision
        self.rhs = [None, W1, W2, R]
        self.L = L
        self.psi_struct = (list(psi.inds), list(psi.blocks), list(psi.offsets))
        dev = psi.data.device
        self.plans, self.outs = [], []
        x = L
        for i, ((a, b, c), T) in enumerate(zip(steps, [psi, W1, W2, R])):
            last = i == len(steps) - 1
            p = ContractionPlan(x, a, T, b, c) if last else get_plan(x, a, T, b, c)
            self.plans.append(p)
            if not last:
                o = BlockSparseTensor(list(p.indsR), list(p.blocksR), list(p.offsetsR),
                                      torch.empty(max(p.nnzR, 1), dtype=torch.float64, device=dev)[:p.nnzR])
                self.outs.append(o)
                x = o
        p = self.plans[-1]
        if sorted(map(tuple, p.blocksR)) != sorted(map(tuple, psi.blocks)) or p.nnzR != psi.nnz:
            raise ValueError("H_eff does not map psi's block structure onto itself")
        where = {tuple(b): o for b, o in zip(psi.blocks, psi.offsets)}
        p.set_output_offsets([where[tuple(b)] for b in p.blocksR])
        self.n = psi.nnz

    def apply(self, x, out):
        """out = H_eff x (x, out: flat psi-ordered device data)."""
        psi = BlockSparseTensor(*self.psi_struct, x)
        cur = self.L
        p = self.plans[-1]
        res = BlockSparseTensor(list(p.indsR), list(p.blocksR), list(p.offsetsR), out)
        dests = self.outs + [res]
        for (a, b, c), T, pl, o in zip(self.steps, [psi] + self.rhs[1:], self.plans, dests):
            contract_blocksparse(cur, a, T, b, c, precision=self.precision, plan=pl, out=o)
            cur = o
        return out


class LanczosResult:
    def __init__(self, value, vector, residual, alpha, beta, krylovdim):
        self.value, self.vector, self.residual = value, vector, residual
        self.alpha, self.beta, self.krylovdim = alpha, beta, krylovdim


class Lanczos:
    """Krylov basis construction for one operator and vector length, reusable (and
    capturable) across calls: `run(v0)` returns the lowest Ritz pair ("SR").  With
    device_solve the krylovdim x krylovdim tridiagonal problem and the Ritz vector are
    computed on the device too (nd_tridiag_lowest_f64), so `enqueue()` is a whole solve
    with no host synchronisation."""

    def __init__(self, apply, n, krylovdim=10, device=0, graph=False, device_solve=False):
        import torch
        self.apply, self.n, self.k, self.graph = apply, n, int(krylovdim), graph
        self.device_solve = device_solve
        if self.k + 1 > 32:
            raise ValueError("krylovdim must be at most 31 (the library's basis operations take 32 vectors)")
        dev = torch.device("cuda", device)
        f64 = dict(dtype=torch.float64, device=dev)
        self.V = torch.zeros((self.k + 1, n), **f64)         # basis, one vector per row (ldv = n)
        self.w = torch.empty(n, **f64)
        self.coef = torch.empty((2, self.k + 1), **f64)       # Gram-Schmidt coefficients of the two passes
        self.alpha = torch.zeros(self.k, **f64)
        self.beta = torch.zeros(self.k, **f64)
        self.s = torch.empty(1, **f64)
        self.start = torch.empty(n, **f64)
        self.value = torch.zeros(1, **f64)                    # device solve: lowest Ritz value
        self.y = torch.zeros(self.k, **f64)                   # and its coefficients in the basis
        self.x = torch.empty(n, **f64)                        # the Ritz vector
        self.device = device
        self._graph = None

    def _body(self):
        h = handle(self.device)
        n, V, w = self.n, self.V, self.w
        h.call("nd_vec_norm_f64", n, _p(self.start), _p(self.s))
        h.call("nd_vec_scale_f64", n, _p(self.start), _p(V), 1.0, _p(self.s), 1)           # V0 = start / |start|
        for j in range(self.k):
            self.apply(V[j], w)
            for sweep in range(2):                                                       # full re-orthogonalisation
                c = self.coef[sweep]
                h.call("nd_vec_dots_f64", n, j + 1, _p(V), n, _p(w), _p(c))              # c = V[:j+1] w
                h.call("nd_vec_update_f64", n, j + 1, _p(V), n, _p(c), -1.0, _p(w))       # w -= V[:j+1]^T c
            a = self.alpha[j:j + 1]
            h.call("nd_vec_add_f64", 1, _p(self.coef[0], j), _p(a), 1.0, 0.0)             # alpha_j = c0_j + c1_j
            h.call("nd_vec_add_f64", 1, _p(self.coef[1], j), _p(a), 1.0, 1.0)
            h.call("nd_vec_norm_f64", n, _p(w), _p(self.beta, j))                          # beta_j = |w|
            h.call("nd_vec_scale_f64", n, _p(w), _p(V, (j + 1) * n), 1.0, _p(self.beta, j), 1)   # V_{j+1} = w / beta_j

    def _solve_device(self):
        h = handle(self.device)
        h.call("nd_tridiag_lowest_f64", self.k, _p(self.alpha), _p(self.beta), _p(self.value), _p(self.y))
        h.call("nd_vec_scale_f64", self.n, _p(self.V), _p(self.x), 0.0, None, 0)                   # x = 0
        h.call("nd_vec_update_f64", self.n, self.k, _p(self.V), self.n, _p(self.y), 1.0, _p(self.x))  # x = V^T y

    def enqueue(self):
        """The whole solve from self.start (basis, tridiagonal eigenpair, Ritz vector into
        self.x, value into self.value): library launches only, no synchronisation."""
        self._body()
        self._solve_device()

    def run(self, v0):
        import torch
        h = handle(self.device)
        h.call("nd_vec_scale_f64", self.n, _p(v0), _p(self.start), 1.0, None, 0)
        if self.device_solve:
            if not self.graph:
                self.enqueue()
            else:
                if self._graph is None:
                    s = torch.cuda.Stream()
                    s.wait_stream(torch.cuda.current_stream())
                    with torch.cuda.stream(s):
                        self.enqueue()                  # warm-up outside capture: builds every cache
                    torch.cuda.current_stream().wait_stream(s)
                    self._graph = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(self._graph):
                        self.enqueue()
                self._graph.replay()
            b = self.beta.cpu().numpy()
            y = self.y.cpu().numpy()
            return LanczosResult(float(self.value.item()), self.x, float(abs(b[-1] * y[-1])),
                                 self.alpha.cpu().numpy(), b, self.k)
        if not self.graph:
            self._body()
        else:
            if self._graph is None:
                s = torch.cuda.Stream()
                s.wait_stream(torch.cuda.current_stream())
                with torch.cuda.stream(s):
                    self._body()                        # warm-up outside capture: builds every cache
                torch.cuda.current_stream().wait_stream(s)
                self._graph = torch.cuda.CUDAGraph()
                with torch.cuda.graph(self._graph):
                    self._body()
            self._graph.replay()
        a = self.alpha.cpu().numpy()
        b = self.beta.cpu().numpy()
        T = np.diag(a) + np.diag(b[:-1], 1) + np.diag(b[:-1], -1)
        vals, vecs = np.linalg.eigh(T)
        y = torch.from_numpy(np.ascontiguousarray(vecs[:, 0])).to(self.V.device)
        x = torch.empty(self.n, dtype=torch.float64, device=self.V.device)
        h = handle(self.device)
        h.call("nd_vec_scale_f64", self.n, _p(self.V), _p(x), 0.0, None, 0)                # x = 0
        h.call("nd_vec_update_f64", self.n, self.k, _p(self.V), self.n, _p(y), 1.0, _p(x))  # x = V[:k]^T y
        return LanczosResult(float(vals[0]), x, float(abs(b[-1] * y[-1].item())), a, b, self.k)


def lanczos(apply, v0, krylovdim=10, graph=False):
    """Lowest Ritz pair of the operator `apply(x, out)` from a Krylov basis built on v0."""
    return Lanczos(apply, v0.numel(), krylovdim, v0.device.index or 0, graph).run(v0)


class SweepStep:
    """One two-site update of a DMRG sweep on the device: the lowest eigenpair of H_eff
    by Lanczos (cached contraction plans, the small tridiagonal problem on the device),
    the Ritz vector matricized to (row dims) x (column dims) and its truncated blockwise
    SVD (SvdPlan).  Every step is library launches with no host synchronisation, so with
    graph=True the whole update is captured once into one CUDA graph and replayed; the
    energy, the factors and the kept dimensions are read after the replay (result()).
    The reference performs this update in ITensorMPS (outside the repository) on
    NDTensors' contract, svd and truncate! (NDTensors/src/blocksparse/linearalgebra.jl:45-215)."""

    def __init__(self, L, W1, W2, R, psi: BlockSparseTensor, steps, qinds, row_dims, col_dims, krylovdim=10,
                 precision="ozaki", graph=True, **svd_kwargs):
        from .linalg import MatricizePlan, SvdPlan
        self.op = HeffOperator(L, W1, W2, R, psi, steps, precision=precision)
        dev = psi.data.device.index or 0
        self.lz = Lanczos(self.op.apply, self.op.n, krylovdim, dev, device_solve=True)
        self.psi_struct = (list(psi.inds), list(psi.blocks), list(psi.offsets))
        self.mat = MatricizePlan(psi, qinds, row_dims, col_dims)
        self.svd = SvdPlan(self.mat.M, **svd_kwargs)
        self.graph = graph
        self._graph = None
        self.device = dev

    def _enqueue(self):
        self.lz.enqueue()
        M = self.mat.run(self.lz.x)
        self.svd.run(M)

    def run(self, v0):
        """Enqueue (or replay) one update from the start vector v0 (psi-ordered data)."""
        import torch
        handle(self.device).call("nd_vec_scale_f64", self.lz.n, _p(v0), _p(self.lz.start), 1.0, None, 0)
        if not self.graph:
            self._enqueue()
            return
        if self._graph is None:
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self._enqueue()                         # warm-up outside capture: builds every cache
            torch.cuda.current_stream().wait_stream(s)
            torch.cuda.synchronize()
            self._graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(self._graph):
                self._enqueue()
        self._graph.replay()

    def result(self):
        """(energy, Ritz vector, svd result as svd() returns it or None) after run()."""
        return float(self.lz.value.item()), self.lz.x, self.svd.result()
