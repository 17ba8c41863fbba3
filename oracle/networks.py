"""Seeded synthetic workloads for the contraction path (oracle side).

No external dataset is involved: every tensor is drawn from numpy's PCG64
generator with a recorded seed, so the same inputs are produced on any host.

Workloads (index conventions are this project's; arrows make every QN tensor
flux-0):
  dense_pair        A(a,s,b) * B(b,t,c) -> C(a,s,t,c), then permute to (s,a,c,t)
  dense_heff        L(lo,wl,l) psi(l,s1,s2,r) W1(wl,s1o,s1,wm) W2(wm,s2o,s2,wr) R(ro,wr,r)
                    contracted in the order L, psi, W1, W2, R
  qn_pair           A(l,s,r) * B(r,t,c) over r, U(1) charges, flux 0
  qn_heff           the two-site H_eff network with QN block sparsity

The XXZ MPO (Jz, Jxy) is the standard lower-triangular w = 5 form built from the
spin-1/2 operators of src/lib/SiteTypes/src/sitetypes/qubit.jl:433-449
(Sz = diag(1/2, -1/2), S+ = |up><dn|, S- = |dn><up|); spin-1/2 sector charges
are 2*Sz = +1 / -1 (src/lib/SiteTypes/src/sitetypes/spinhalf.jl:27).
"""
from __future__ import annotations

import numpy as np

from .blocksparse import BlockSparseTensor, blockoffsets
from .qn import QNIndex, nzblocks

SZ = np.array([[0.5, 0.0], [0.0, -0.5]])
SP = np.array([[0.0, 1.0], [0.0, 0.0]])
SM = np.array([[0.0, 0.0], [1.0, 0.0]])
ID = np.eye(2)


def sector_dims(chi, sigma=3.0, qmax=8, dmin=8):
    """Sector dims d_q = round(chi * phi(q; 0, sigma) / sum(phi)), at least dmin,
    remainder to q = 0.  Returns [(q, d_q)] for q = -qmax..qmax (ascending)."""
    qs = np.arange(-qmax, qmax + 1)
    phi = np.exp(-qs.astype(np.float64) ** 2 / (2.0 * sigma * sigma))
    d = np.round(chi * phi / phi.sum()).astype(np.int64)
    d = np.maximum(d, dmin)
    d[qmax] += chi - int(d.sum())
    if d[qmax] < 1:
        raise ValueError(f"chi = {chi} leaves no states for the q = 0 sector ({2 * qmax + 1} sectors, min {dmin})")
    return [(int(q), int(x)) for q, x in zip(qs, d)]


def xxz_mpo_dense(jz=1.0, jxy=1.0):
    """W[wl, s', s, wr] of the lower-triangular w = 5 XXZ MPO."""
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


# link basis grouped by charge: states (0,3,4) carry 0, state 1 carries +2, state 2 carries -2
MPO_LINK_ORDER = [0, 3, 4, 1, 2]
MPO_LINK_SECTORS = ((0, 3), (2, 1), (-2, 1))
SPIN_SECTORS = ((1, 1), (-1, 1))


def dense_pair(seed=0, a=128, s=2, b=128, t=2, c=128):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((a, s, b))
    B = rng.standard_normal((b, t, c))
    return A, B


def dense_heff(chi=1024, d=2, w=5, seed=1, jz=1.0, jxy=1.0):
    rng = np.random.default_rng(seed)
    sc = 1.0 / np.sqrt(chi)
    L = rng.standard_normal((chi, w, chi)) * sc
    psi = rng.standard_normal((chi, d, d, chi)) * sc
    R = rng.standard_normal((chi, w, chi)) * sc
    W = xxz_mpo_dense(jz, jxy)
    return dict(L=L, psi=psi, W1=W.copy(), W2=W.copy(), R=R)


# labels of the H_eff chain: lo=1, wl=2, l=3, s1=4, s2=5, r=6, s1o=7, wm=8, s2o=9, wr=10, ro=11
HEFF_LABELS = dict(L=(1, 2, 3), psi=(3, 4, 5, 6), W1=(2, 7, 4, 8), W2=(8, 9, 5, 10),
                   R=(11, 10, 6), out=(1, 7, 9, 11))


def heff_steps():
    """The four pairwise steps as (left labels, right labels, output labels) in
    ncon form (contracted labels negative), order L, psi, W1, W2, R."""
    return [
        # T1(lo, wl, s1, s2, r) = L(lo, wl, l) psi(l, s1, s2, r)
        ((1, 2, -1), (-1, 4, 5, 6), (1, 2, 4, 5, 6)),
        # T2(lo, s2, r, s1o, wm) = T1(lo, wl, s1, s2, r) W1(wl, s1o, s1, wm)
        ((1, -1, -2, 5, 6), (-1, 7, -2, 8), (1, 5, 6, 7, 8)),
        # T3(lo, r, s1o, s2o, wr) = T2(lo, s2, r, s1o, wm) W2(wm, s2o, s2, wr)
        ((1, -2, 6, 7, -1), (-1, 9, -2, 10), (1, 6, 7, 9, 10)),
        # T4(lo, s1o, s2o, ro) = T3(lo, r, s1o, s2o, wr) R(ro, wr, r)
        ((1, -1, 7, 9, -2), (11, -2, -1), (1, 7, 9, 11)),
    ]


def heff_apply_dense(net, contract):
    """Apply H_eff with a pairwise ``contract(A, la, B, lb, lr)`` callable."""
    st = heff_steps()
    t = contract(net["L"], st[0][0], net["psi"], st[0][1], st[0][2])
    t = contract(t, st[1][0], net["W1"], st[1][1], st[1][2])
    t = contract(t, st[2][0], net["W2"], st[2][1], st[2][2])
    t = contract(t, st[3][0], net["R"], st[3][1], st[3][2])
    return t


def heff_flops_dense(chi, d=2, w=5):
    return (2 * chi * w * chi * d * d * chi          # L psi
            + 2 * chi * d * chi * d * w * w * d      # T1 W1: M=lo*s2*r, K=wl*s1, N=s1o*wm
            + 2 * chi * chi * d * w * d * w * d      # T2 W2
            + 2 * chi * d * d * chi * w * chi)       # T3 R


# ---------------------------------------------------------------------------
# QN block-sparse workloads
# ---------------------------------------------------------------------------

def qn_tensor(rng, qinds, flux=0, scale=1.0):
    blocks = nzblocks(flux, qinds)
    inds = [q.dims for q in qinds]
    offs, nnz = blockoffsets(blocks, inds)
    data = rng.standard_normal(nnz) * scale
    return BlockSparseTensor(inds, blocks, offs, data)


def qn_pair(chi=2048, seed=2, sigma=3.0, qmax=8):
    """A(l,s,r) * B(r,t,c): l Out, s Out, r In in A; r Out, t Out, c In in B."""
    rng = np.random.default_rng(seed)
    sec = tuple(sector_dims(chi, sigma, qmax))
    l = QNIndex(sec, 1, "l")
    s = QNIndex(SPIN_SECTORS, 1, "s")
    r = QNIndex(sec, -1, "r")
    t = QNIndex(SPIN_SECTORS, 1, "t")
    c = QNIndex(sec, -1, "c")
    A = qn_tensor(rng, [l, s, r])
    B = qn_tensor(rng, [r.dag(), t, c])
    return A, B, dict(A=[l, s, r], B=[r.dag(), t, c])


def mpo_qn(jz=1.0, jxy=1.0):
    """QN block-sparse W(wl In, s' Out, s In, wr Out) with link sectors
    {0: 3, +2: 1, -2: 1}; dense entries taken from the lower-triangular MPO."""
    W = xxz_mpo_dense(jz, jxy)[MPO_LINK_ORDER][:, :, :, MPO_LINK_ORDER]
    wl = QNIndex(MPO_LINK_SECTORS, -1, "wl")
    so = QNIndex(SPIN_SECTORS, 1, "so")
    si = QNIndex(SPIN_SECTORS, -1, "si")
    wr = QNIndex(MPO_LINK_SECTORS, 1, "wr")
    qinds = [wl, so, si, wr]
    blocks = nzblocks(0, qinds)
    inds = [q.dims for q in qinds]
    offs, nnz = blockoffsets(blocks, inds)
    T = BlockSparseTensor(inds, blocks, offs, np.zeros(nnz))
    starts = [np.concatenate([[0], np.cumsum(q.dims)[:-1]]) for q in qinds]
    for i, b in enumerate(blocks):
        sl = tuple(slice(int(starts[k][b[k] - 1]), int(starts[k][b[k] - 1]) + inds[k][b[k] - 1])
                   for k in range(4))
        T.blockview(i)[...] = W[sl]
    # every nonzero of W must sit in an allowed block
    assert np.allclose(T.to_dense(), W)
    return T, qinds


def qn_heff(chi=4096, seed=3, sigma=3.0, qmax=8, jz=1.0, jxy=1.0):
    """Two-site H_eff network with U(1) block sparsity (all tensors flux 0).

    psi(l Out, s1 Out, s2 Out, r In); L(lo Out, wl Out, l In);
    W1(wl In, s1o Out, s1 In, wm Out); W2(wm In, s2o Out, s2 In, wr Out);
    R(ro In, wr In, r Out).  Entries of L, R, psi ~ N(0, 1/chi).
    """
    rng = np.random.default_rng(seed)
    sec = tuple(sector_dims(chi, sigma, qmax))
    sc = 1.0 / np.sqrt(chi)
    l = QNIndex(sec, 1, "l")
    r = QNIndex(sec, -1, "r")
    s1 = QNIndex(SPIN_SECTORS, 1, "s1")
    s2 = QNIndex(SPIN_SECTORS, 1, "s2")
    lo = QNIndex(sec, 1, "l", 1)
    ro = QNIndex(sec, -1, "r", 1)
    wl = QNIndex(MPO_LINK_SECTORS, 1, "wl")
    wr = QNIndex(MPO_LINK_SECTORS, -1, "wr")
    psi = qn_tensor(rng, [l, s1, s2, r], 0, sc)
    L = qn_tensor(rng, [lo, wl, l.dag()], 0, sc)
    R = qn_tensor(rng, [ro, wr, r.dag()], 0, sc)
    W, _ = mpo_qn(jz, jxy)
    qinds = dict(psi=[l, s1, s2, r], L=[lo, wl, l.dag()], R=[ro, wr, r.dag()])
    return dict(L=L, psi=psi, W1=W, W2=W, R=R, qinds=qinds)
