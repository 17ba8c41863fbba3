"""Lanczos eigensolver for an effective Hamiltonian, on the device.

A DMRG sweep solves its local eigenproblem with KrylovKit over the vector-space
interface the reference provides for ITensors
(ext/ITensorsVectorInterfaceExt/ITensorsVectorInterfaceExt.jl:5-84: add / add! /
inner / scale / scale!).  Here a vector is the flat FP64 data of a
tensor with a fixed block structure, the VectorInterface operations are torch
ops on that data (`inner`, `norm`, `add_`, `scale_`), and the operator is a
sequence of library contractions (`HeffOperator`: the two-site H_eff applied as
L * psi, * W1, * W2, * R with cached plans and preallocated intermediates).

`lanczos` builds a Krylov basis of `krylovdim` vectors with full
re-orthogonalisation (classical Gram-Schmidt, twice).  With ``graph=True`` the
whole basis construction -- every matvec and every orthogonalisation -- is
captured once into one CUDA graph (torch.cuda.graph; the library detects the
capture and only launches kernels) and replayed; the krylovdim x krylovdim
tridiagonal problem is then solved on the host.
"""
from __future__ import annotations

import numpy as np

from .contract import contract_blocksparse, get_plan
from .tensors import BlockSparseTensor


def inner(x, y):
    """VectorInterface.inner on flat real data (a device scalar)."""
    return (x * y).sum()


def norm(x):
    import torch
    return torch.linalg.vector_norm(x)


def scale_(x, a):
    """VectorInterface.scale!(x, a)."""
    return x.mul_(a)


def add_(y, x, a=1.0):
    """VectorInterface.add!(y, x, a): y += a x."""
    return y.add_(x, alpha=a)


class HeffOperator:
    """x -> H_eff x for the two-site network (L, W1, W2, R) on a fixed psi structure.

    Plans and the three intermediates are built once; the result is gathered back
    into psi's block order (the plan lists output blocks in first-appearance order),
    so the operator maps the vector space onto itself and can be captured.
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
        for (a, b, c), T in zip(steps, [psi, W1, W2, R]):
            p = get_plan(x, a, T, b, c)
            o = BlockSparseTensor(list(p.indsR), list(p.blocksR), list(p.offsetsR),
                                  torch.empty(max(p.nnzR, 1), dtype=torch.float64, device=dev)[:p.nnzR])
            self.plans.append(p)
            self.outs.append(o)
            x = o
        out = self.outs[-1]
        if sorted(map(tuple, out.blocks)) != sorted(map(tuple, psi.blocks)) or out.nnz != psi.nnz:
            raise ValueError("H_eff does not map psi's block structure onto itself")
        # element gather: psi-ordered data = out.data[index]
        index = np.empty(psi.nnz, dtype=np.int64)
        where = {tuple(b): o for b, o in zip(out.blocks, out.offsets)}
        for b, off in zip(psi.blocks, psi.offsets):
            n = int(np.prod(psi.blockdims(b)))
            src = where[tuple(b)]
            index[off:off + n] = np.arange(src, src + n)
        self.identity = bool(np.array_equal(index, np.arange(psi.nnz)))
        self.index = torch.from_numpy(index).to(dev)
        self.n = psi.nnz

    def apply(self, x, out):
        """out = H_eff x (x, out: flat psi-ordered device data)."""
        import torch
        psi = BlockSparseTensor(*self.psi_struct, x)
        cur = self.L
        for (a, b, c), T, p, o in zip(self.steps, [psi] + self.rhs[1:], self.plans, self.outs):
            if T is psi:
                contract_blocksparse(cur, a, psi, b, c, precision=self.precision, plan=p, out=o)
            else:
                contract_blocksparse(cur, a, T, b, c, precision=self.precision, plan=p, out=o)
            cur = o
        if self.identity:
            out.copy_(self.outs[-1].data)
        else:
            torch.index_select(self.outs[-1].data, 0, self.index, out=out)
        return out


class LanczosResult:
    def __init__(self, value, vector, residual, alpha, beta, krylovdim):
        self.value, self.vector, self.residual = value, vector, residual
        self.alpha, self.beta, self.krylovdim = alpha, beta, krylovdim


class Lanczos:
    """Krylov basis construction for one operator and vector length, reusable (and
    capturable) across calls: `run(v0)` returns the lowest Ritz pair ("SR")."""

    def __init__(self, apply, n, krylovdim=10, device=0, graph=False):
        import torch
        self.apply, self.n, self.k, self.graph = apply, n, int(krylovdim), graph
        dev = torch.device("cuda", device)
        f64 = dict(dtype=torch.float64, device=dev)
        self.V = torch.zeros((self.k + 1, n), **f64)
        self.w = torch.empty(n, **f64)
        self.coef = torch.empty(self.k + 1, **f64)
        self.alpha = torch.zeros(self.k, **f64)
        self.beta = torch.zeros(self.k, **f64)
        self.start = torch.empty(n, **f64)
        self._graph = None

    def _body(self):
        import torch
        V, w, coef = self.V, self.w, self.coef
        V[0].copy_(self.start)
        V[0].div_(torch.linalg.vector_norm(V[0]))
        for j in range(self.k):
            self.apply(V[j], w)
            basis = V[:j + 1]
            for sweep in range(2):                      # full re-orthogonalisation
                torch.mv(basis, w, out=coef[:j + 1])
                if sweep == 0:
                    self.alpha[j:j + 1].copy_(coef[j:j + 1])
                else:
                    self.alpha[j:j + 1].add_(coef[j:j + 1])
                w.addmv_(basis.t(), coef[:j + 1], alpha=-1.0)
            self.beta[j:j + 1].copy_(torch.linalg.vector_norm(w).reshape(1))
            torch.div(w, self.beta[j], out=V[j + 1])

    def run(self, v0):
        import torch
        self.start.copy_(v0)
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
        y = vecs[:, 0]
        x = torch.mv(self.V[:self.k].t(), torch.from_numpy(y).to(self.V.device))
        return LanczosResult(float(vals[0]), x, float(abs(b[-1] * y[-1])), a, b, self.k)


def lanczos(apply, v0, krylovdim=10, graph=False):
    """Lowest Ritz pair of the operator `apply(x, out)` from a Krylov basis built on v0."""
    return Lanczos(apply, v0.numel(), krylovdim, v0.device.index or 0, graph).run(v0)
