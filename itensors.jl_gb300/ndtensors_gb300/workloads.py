"""Seeded synthetic workloads of the contraction path (host numpy data).

No external dataset is involved: every tensor is drawn from numpy's PCG64
generator with a recorded seed, so every host produces the same inputs.

  dense_pair   A(a,s,b) * B(b,t,c) -> C(a,s,t,c), then permute to (s,a,c,t)
  dense_heff   L(lo,wl,l) psi(l,s1,s2,r) W1(wl,s1o,s1,wm) W2(wm,s2o,s2,wr) R(ro,wr,r)
  qn_pair      A(l,s,r) * B(r,t,c) over r with U(1) charges, flux 0
  qn_heff      the two-site H_eff network with U(1) block sparsity

QN structure follows NDTensors/ITensors: sectors are (charge, dim) with an arrow,
block lists are CartesianIndices order (first index fastest) filtered by flux
(NDTensors/src/blocksparse/blockdims.jl:104-106, src/qn/qnindexset.jl:9-18).
The XXZ MPO is the lower-triangular w = 5 form built from the spin-1/2
operators of src/lib/SiteTypes/src/sitetypes/qubit.jl:433-449; spin sectors
carry 2*Sz = +1 / -1 (src/lib/SiteTypes/src/sitetypes/spinhalf.jl:27).
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np

SZ = np.array([[0.5, 0.0], [0.0, -0.5]])
SP = np.array([[0.0, 1.0], [0.0, 0.0]])
SM = np.array([[0.0, 0.0], [1.0, 0.0]])
ID = np.eye(2)
SPIN_SECTORS = ((1, 1), (-1, 1))
# MPO link basis grouped by charge: states (0, 3, 4) carry 0, state 1 carries +2, state 2 carries -2
MPO_LINK_ORDER = [0, 3, 4, 1, 2]
MPO_LINK_SECTORS = ((0, 3), (2, 1), (-2, 1))


@dataclass
class HostBlockSparse:
    """inds: per dimension the block dims; blocks 1-based; offsets 0-based; data flat FP64."""
    inds: list
    blocks: list
    offsets: list
    data: np.ndarray

    @property
    def nnz(self):
        return int(self.data.size)


def sector_dims(chi, sigma=3.0, qmax=8, dmin=8):
    """d_q = round(chi * phi(q; 0, sigma) / sum phi), at least dmin, remainder to q = 0."""
    qs = np.arange(-qmax, qmax + 1)
    phi = np.exp(-qs.astype(np.float64) ** 2 / (2.0 * sigma * sigma))
    d = np.round(chi * phi / phi.sum()).astype(np.int64)
    d = np.maximum(d, dmin)
    d[qmax] += chi - int(d.sum())
    if d[qmax] < 1:
        raise ValueError(f"chi = {chi} leaves no states for the q = 0 sector ({2 * qmax + 1} sectors, min {dmin})")
    return [(int(q), int(x)) for q, x in zip(qs, d)]


def nzblocks(flux, sectors_arrows):
    """Blocks with the requested flux, first index fastest."""
    ranges = [range(1, len(s) + 1) for s, _ in sectors_arrows]
    out = []
    for t in itertools.product(*reversed(ranges)):
        b = tuple(reversed(t))
        f = sum(a * s[bk - 1][0] for (s, a), bk in zip(sectors_arrows, b))
        if f == flux:
            out.append(b)
    return out


def random_qn(rng, sectors_arrows, flux=0, scale=1.0):
    blocks = nzblocks(flux, sectors_arrows)
    inds = [tuple(d for _, d in s) for s, _ in sectors_arrows]
    offs, nnz = [], 0
    for b in blocks:
        offs.append(nnz)
        nnz += int(np.prod([inds[k][b[k] - 1] for k in range(len(inds))]))
    return HostBlockSparse(inds, blocks, offs, rng.standard_normal(nnz) * scale)


def xxz_mpo_dense(jz=1.0, jxy=1.0):
    W = np.zeros((5, 2, 2, 5))
    W[0, :, :, 0] = ID
    W[1, :, :, 0] = SP
    W[2, :, :, 0] = SM
    W[3, :, :, 0] = SZ
    W[4, :, :, 1] = 0.5 * jxy * SM
    W[4, :, :, 2] = 0.5 * jxy * SP
    W[4, :, :, 3] = jz * SZ
    W[4, :, :, 4] = ID
    return W


def mpo_qn(jz=1.0, jxy=1.0):
    """W(wl In, s' Out, s In, wr Out), link sectors {0: 3, +2: 1, -2: 1}."""
    W = xxz_mpo_dense(jz, jxy)[MPO_LINK_ORDER][:, :, :, MPO_LINK_ORDER]
    sa = [(MPO_LINK_SECTORS, -1), (SPIN_SECTORS, 1), (SPIN_SECTORS, -1), (MPO_LINK_SECTORS, 1)]
    blocks = nzblocks(0, sa)
    inds = [tuple(d for _, d in s) for s, _ in sa]
    starts = [np.concatenate([[0], np.cumsum(i)[:-1]]).astype(int) for i in inds]
    offs, chunks, nnz = [], [], 0
    for b in blocks:
        sl = tuple(slice(starts[k][b[k] - 1], starts[k][b[k] - 1] + inds[k][b[k] - 1]) for k in range(4))
        blk = W[sl]
        offs.append(nnz)
        chunks.append(blk.reshape(-1, order="F"))
        nnz += blk.size
    return HostBlockSparse(inds, blocks, offs, np.concatenate(chunks))


def dense_pair(seed=0, a=128, s=2, b=128, t=2, c=128):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((a, s, b)), rng.standard_normal((b, t, c))


def dense_heff(chi=1024, d=2, w=5, seed=1, jz=1.0, jxy=1.0):
    rng = np.random.default_rng(seed)
    sc = 1.0 / np.sqrt(chi)
    L = rng.standard_normal((chi, w, chi)) * sc
    psi = rng.standard_normal((chi, d, d, chi)) * sc
    R = rng.standard_normal((chi, w, chi)) * sc
    W = xxz_mpo_dense(jz, jxy)
    return dict(L=L, psi=psi, W1=W.copy(), W2=W.copy(), R=R)


def heff_steps():
    """(left labels, right labels, output labels) of the four pairwise steps, order
    L, psi, W1, W2, R; contracted labels are negative (ncon form).
      T1(lo,wl,s1,s2,r)  = L(lo,wl,l) psi(l,s1,s2,r)
      T2(lo,s2,r,s1o,wm) = T1 W1(wl,s1o,s1,wm)
      T3(lo,r,s1o,s2o,wr)= T2 W2(wm,s2o,s2,wr)
      T4(lo,s1o,s2o,ro)  = T3 R(ro,wr,r)"""
    return [
        ((1, 2, -1), (-1, 4, 5, 6), (1, 2, 4, 5, 6)),
        ((1, -1, -2, 5, 6), (-1, 7, -2, 8), (1, 5, 6, 7, 8)),
        ((1, -2, 6, 7, -1), (-1, 9, -2, 10), (1, 6, 7, 9, 10)),
        ((1, -1, 7, 9, -2), (11, -2, -1), (1, 7, 9, 11)),
    ]


def heff_flops_dense(chi, d=2, w=5):
    return (2 * chi * w * chi * d * d * chi + 2 * chi * d * chi * d * w * w * d
            + 2 * chi * chi * d * w * d * w * d + 2 * chi * d * d * chi * w * chi)


def qn_pair(chi=2048, seed=2, sigma=3.0, qmax=8):
    """A(l Out, s Out, r In) * B(r Out, t Out, c In)."""
    rng = np.random.default_rng(seed)
    sec = tuple(sector_dims(chi, sigma, qmax))
    A = random_qn(rng, [(sec, 1), (SPIN_SECTORS, 1), (sec, -1)])
    B = random_qn(rng, [(sec, 1), (SPIN_SECTORS, 1), (sec, -1)])
    return A, B


def qn_heff(chi=4096, seed=3, sigma=3.0, qmax=8, jz=1.0, jxy=1.0):
    """Two-site H_eff network, all tensors flux 0.

    psi(l Out, s1 Out, s2 Out, r In); L(lo Out, wl Out, l In); R(ro In, wr In, r Out);
    W1 = W2 = W(wl In, s' Out, s In, wr Out).  Entries of L, R, psi ~ N(0, 1/chi).
    """
    rng = np.random.default_rng(seed)
    sec = tuple(sector_dims(chi, sigma, qmax))
    sc = 1.0 / np.sqrt(chi)
    psi = random_qn(rng, [(sec, 1), (SPIN_SECTORS, 1), (SPIN_SECTORS, 1), (sec, -1)], 0, sc)
    L = random_qn(rng, [(sec, 1), (MPO_LINK_SECTORS, 1), (sec, -1)], 0, sc)
    R = random_qn(rng, [(sec, -1), (MPO_LINK_SECTORS, -1), (sec, 1)], 0, sc)
    W = mpo_qn(jz, jxy)
    return dict(L=L, psi=psi, W1=W, W2=W, R=R, sectors=sec)
