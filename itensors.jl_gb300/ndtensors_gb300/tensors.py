"""Device tensors with NDTensors' storage conventions.

DenseTensor        dims + one column-major FP64 vector (NDTensors Dense, dense/dense.jl:5-18)
BlockSparseTensor  per-dimension block dims + ordered nonzero blocks (1-based) +
                   0-based offsets into one FP64 vector (BlockSparse,
                   blocksparse/blocksparse.jl:5-13; BlockOffsets, blockoffsets.jl:11)

Data live in torch CUDA float64 tensors; torch is only the allocator here.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


def _torch():
    import torch
    return torch


def _prod(xs):
    p = 1
    for x in xs:
        p *= int(x)
    return p


@dataclass
class DenseTensor:
    dims: tuple
    data: object          # torch.float64 CUDA 1-D, column-major

    @property
    def rank(self):
        return len(self.dims)

    @property
    def nnz(self):
        return _prod(self.dims)

    @classmethod
    def empty(cls, dims, device=0):
        torch = _torch()
        return cls(tuple(int(d) for d in dims),
                   torch.empty(max(1, _prod(dims)), dtype=torch.float64, device=f"cuda:{device}")[:_prod(dims)])

    @classmethod
    def from_numpy(cls, arr, device=0):
        torch = _torch()
        arr = np.asarray(arr, dtype=np.float64)
        flat = np.ascontiguousarray(arr.reshape(-1, order="F"))
        return cls(tuple(arr.shape), torch.from_numpy(flat).to(f"cuda:{device}"))

    def to_numpy(self):
        return self.data.detach().cpu().numpy().reshape(self.dims, order="F")

    def ptr(self):
        return self.data.data_ptr()


def blockoffsets(blocks, inds):
    """Offsets in list order (NDTensors/src/blocksparse/blockoffsets.jl:70-79)."""
    offs, nnz = [], 0
    for b in blocks:
        offs.append(nnz)
        nnz += _prod(inds[k][b[k] - 1] for k in range(len(inds)))
    return offs, nnz


@dataclass
class BlockSparseTensor:
    inds: list            # per dimension: tuple of block dims
    blocks: list          # list of 1-based tuples, storage order
    offsets: list
    data: object          # torch.float64 CUDA 1-D
    _key: tuple = field(default=None, repr=False)
    _desc: object = field(default=None, repr=False)

    @property
    def rank(self):
        return len(self.inds)

    @property
    def nnz(self):
        return int(self.data.numel())

    @property
    def nnzblocks(self):
        return len(self.blocks)

    def blockdims(self, block):
        return tuple(self.inds[k][block[k] - 1] for k in range(self.rank))

    def structure_key(self):
        if self._key is None:
            self._key = (tuple(tuple(i) for i in self.inds), tuple(tuple(b) for b in self.blocks),
                         tuple(self.offsets))
        return self._key

    @classmethod
    def empty(cls, inds, blocks, device=0):
        torch = _torch()
        inds = [tuple(int(x) for x in i) for i in inds]
        blocks = [tuple(int(x) for x in b) for b in blocks]
        offs, nnz = blockoffsets(blocks, inds)
        return cls(inds, blocks, offs, torch.empty(max(nnz, 1), dtype=torch.float64,
                                                   device=f"cuda:{device}")[:nnz])

    @classmethod
    def from_oracle(cls, t, device=0):
        """From an oracle.blocksparse.BlockSparseTensor (host numpy)."""
        torch = _torch()
        return cls([tuple(i) for i in t.inds], [tuple(b) for b in t.blocks], list(t.offsets),
                   torch.from_numpy(np.ascontiguousarray(t.data, dtype=np.float64)).to(f"cuda:{device}"))

    @classmethod
    def from_host(cls, t, device=0):
        """From a workloads.HostBlockSparse (host numpy)."""
        torch = _torch()
        return cls([tuple(i) for i in t.inds], [tuple(b) for b in t.blocks], list(t.offsets),
                   torch.from_numpy(np.ascontiguousarray(t.data, dtype=np.float64)).to(f"cuda:{device}"))

    def data_numpy(self):
        return self.data.detach().cpu().numpy()

    def blockview(self, i):
        b = self.blocks[i]
        d = self.blockdims(b)
        n = _prod(d)
        return self.data[self.offsets[i]:self.offsets[i] + n]

    def set_desc_arrays(self, blocks, offsets):
        """Build the C-ABI descriptor from block and offset arrays the caller already has
        (int32 rank-major block numbers, int64 offsets) instead of from the lists."""
        import ctypes as C
        from ._lib import BsDesc
        nb = np.array([len(i) for i in self.inds], dtype=np.int32)
        bd = np.array([d for i in self.inds for d in i], dtype=np.int64)
        bl = np.ascontiguousarray(blocks, dtype=np.int32) if len(self.blocks) else np.zeros(1, np.int32)
        of = np.ascontiguousarray(offsets, dtype=np.int64) if len(self.offsets) else np.zeros(1, np.int64)
        P32, P64 = C.POINTER(C.c_int32), C.POINTER(C.c_int64)
        d = BsDesc(self.rank, nb.ctypes.data_as(P32), bd.ctypes.data_as(P64), len(self.blocks),
                   bl.ctypes.data_as(P32), of.ctypes.data_as(P64))
        d._keep = (nb, bd, bl, of)
        self._desc = d

    def desc(self):
        """nd_bs_desc for the C ABI (arrays built once per tensor and kept on it)."""
        import ctypes as C
        from ._lib import BsDesc
        cached = getattr(self, "_desc", None)
        if cached is not None:
            return cached
        nb = np.array([len(i) for i in self.inds], dtype=np.int32)
        bd = np.array([d for i in self.inds for d in i], dtype=np.int64)
        bl = np.asarray(self.blocks, dtype=np.int32).reshape(-1) if self.blocks else np.zeros(1, np.int32)
        of = np.asarray(self.offsets, dtype=np.int64) if self.offsets else np.zeros(1, np.int64)
        P32, P64 = C.POINTER(C.c_int32), C.POINTER(C.c_int64)
        d = BsDesc(self.rank, nb.ctypes.data_as(P32), bd.ctypes.data_as(P64), len(self.blocks),
                   bl.ctypes.data_as(P32), of.ctypes.data_as(P64))
        d._keep = (nb, bd, bl, of)
        self._desc = d
        return d


@dataclass
class DiagBlockSparseTensor:
    """DiagBlockSparse storage (NDTensors/src/blocksparse/diagblocksparse.jl): block-diagonal
    blocks (every block number equal), each storing only its diagonal, min(blockdims)
    entries, at `offsets` into one flat vector."""
    inds: list
    blocks: list
    offsets: list
    data: object          # torch.float64 CUDA 1-D

    @property
    def rank(self):
        return len(self.inds)

    def blockdims(self, block):
        return tuple(self.inds[k][block[k] - 1] for k in range(self.rank))

    @classmethod
    def from_diagonals(cls, inds, blocks, diags):
        """From per-block diagonal vectors (torch CUDA tensors), in block order."""
        torch = _torch()
        for b in blocks:
            if len(set(b)) != 1:
                raise ValueError("DiagBlockSparse blocks must be block diagonal (all block numbers equal)")
        offs, o = [], 0
        for d in diags:
            offs.append(o)
            o += int(d.numel())
        data = torch.cat([d.reshape(-1).to(torch.float64) for d in diags]) if diags else torch.empty(0)
        return cls([tuple(i) for i in inds], [tuple(b) for b in blocks], offs, data)

    def dense(self):
        """The equal-structure BlockSparseTensor with the diagonals expanded, as NDTensors'
        dense(D) conversion (diag/tensoralgebra/contract.jl:103-214): a library memset and
        one strided scatter of every diagonal (element i of block b to (i, i, ..., i))."""
        import ctypes as C
        from ._lib import BlockCopy, handle
        torch = _torch()
        offs, nnz = blockoffsets(self.blocks, self.inds)
        out = torch.empty(max(nnz, 1), dtype=torch.float64, device=self.data.device)[:nnz]
        h = handle(self.data.device.index or 0)
        if nnz:
            h.call("nd_memset0", C.c_void_p(out.data_ptr()), 8 * nnz)
        copies = []
        for b, o, do in zip(self.blocks, offs, self.offsets):
            dims = self.blockdims(b)
            k = min(dims) if dims else 1
            stride, s = 0, 1                          # column-major offset step of (i, i, ..., i)
            for d in dims:
                stride += s
                s *= d
            c = BlockCopy()
            c.src_off, c.dst_off, c.rank = do, o, 1
            c.dims[0], c.src_strides[0], c.dst_strides[0] = k, 1, stride
            copies.append(c)
        if copies and nnz:
            arr = (BlockCopy * len(copies))(*copies)
            h.call("nd_block_copy_f64", len(copies), arr, C.c_void_p(self.data.data_ptr()), C.c_void_p(out.data_ptr()))
        return BlockSparseTensor(list(self.inds), list(self.blocks), offs, out)
