"""Contraction adjoint (rrule) and gradients of the H_eff energy (GPU).

Gradient of E = <psi|H_eff|psi> / <psi|psi> with respect to psi and W1 on the dense
two-site network at chi = 512 (d = 2, w = 5), from the hand-written adjoint chained
by torch autograd, checked against central finite differences (h = 1e-6, FP64
evaluations) on 64 random unit directions each (bar: 1e-6 relative), and against
an independent oracle gradient (numpy reverse mode, bar 1e-10 / 1e-8 split).
"""
import numpy as np
import pytest

from oracle import dense as odense
from oracle import networks
from oracle.adjoint import contract_pullback

pytestmark = pytest.mark.gpu


def _energy_fn(nd, net, precision):
    import torch
    steps = networks.heff_steps()
    dev = torch.device("cuda")
    fl = lambda a: torch.from_numpy(np.ascontiguousarray(a.reshape(-1, order="F"))).to(dev)
    shapes = {k: net[k].shape for k in ("L", "psi", "W1", "W2", "R")}
    L, W2, R = fl(net["L"]), fl(net["W2"]), fl(net["R"])
    S = nd.dense_structure

    def energy(psi, w1):
        t = nd.contract_autograd(L, S(shapes["L"]), steps[0][0], psi, S(shapes["psi"]), steps[0][1], steps[0][2], precision)
        d1 = [shapes["L"][0], shapes["L"][1], shapes["psi"][1], shapes["psi"][2], shapes["psi"][3]]
        t = nd.contract_autograd(t, S(d1), steps[1][0], w1, S(shapes["W1"]), steps[1][1], steps[1][2], precision)
        d2 = [d1[0], d1[3], d1[4], shapes["W1"][1], shapes["W1"][3]]
        t = nd.contract_autograd(t, S(d2), steps[2][0], W2, S(shapes["W2"]), steps[2][1], steps[2][2], precision)
        d3 = [d2[0], d2[2], d2[3], shapes["W2"][1], shapes["W2"][3]]
        t = nd.contract_autograd(t, S(d3), steps[3][0], R, S(shapes["R"]), steps[3][1], steps[3][2], precision)
        return torch.dot(psi, t) / torch.dot(psi, psi)

    return energy, fl


def _oracle_grads(net):
    """Reverse mode on the CPU oracle: dE/dpsi and dE/dW1."""
    st = networks.heff_steps()
    L, psi, W1, W2, R = (net[k] for k in ("L", "psi", "W1", "W2", "R"))
    t1 = odense.contract(L, st[0][0], psi, st[0][1], st[0][2])
    t2 = odense.contract(t1, st[1][0], W1, st[1][1], st[1][2])
    t3 = odense.contract(t2, st[2][0], W2, st[2][1], st[2][2])
    t4 = odense.contract(t3, st[3][0], R, st[3][1], st[3][2])
    nn = float(np.sum(psi * psi))
    E = float(np.sum(psi * t4)) / nn
    y4 = psi / nn
    g3, _ = contract_pullback(t3, st[3][0], R, st[3][1], st[3][2], y4)
    g2, _ = contract_pullback(t2, st[2][0], W2, st[2][1], st[2][2], g3)
    g1, gW1 = contract_pullback(t1, st[1][0], W1, st[1][1], st[1][2], g2)
    _, gpsi = contract_pullback(L, st[0][0], psi, st[0][1], st[0][2], g1)
    gpsi = gpsi + t4 / nn - 2.0 * E * psi / nn
    return E, gpsi, gW1


@pytest.fixture(scope="module")
def net():
    return networks.dense_heff(chi=512, seed=31)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("ozaki", 1e-8)])
def test_gradient_vs_oracle_and_fd(nd, net, precision, tol):
    import torch
    energy, fl = _energy_fn(nd, net, precision)
    psi = fl(net["psi"]).clone().requires_grad_(True)
    w1 = fl(net["W1"]).clone().requires_grad_(True)
    E = energy(psi, w1)
    E.backward()
    gpsi = psi.grad.detach().cpu().numpy()
    gw1 = w1.grad.detach().cpu().numpy()
    E0, ogpsi, ogw1 = _oracle_grads(net)
    assert abs(E.item() - E0) <= 1e-10 * abs(E0) + 1e-14
    assert odense.rel_frobenius_error(gpsi, ogpsi.reshape(-1, order="F")) <= tol
    assert odense.rel_frobenius_error(gw1, ogw1.reshape(-1, order="F")) <= tol
    # central finite differences with FP64 evaluations, 64 random unit directions per argument
    fd_energy, _ = _energy_fn(nd, net, "fp64")
    rng = np.random.default_rng(99)
    h = 1e-6
    with torch.no_grad():
        p0, w0 = psi.detach(), w1.detach()
        for arg, g in (("psi", gpsi), ("w1", gw1)):
            base = p0 if arg == "psi" else w0
            worst = 0.0
            for _ in range(64):
                d = rng.standard_normal(base.numel())
                d /= np.linalg.norm(d)
                dt = torch.from_numpy(d).to(base.device)
                if arg == "psi":
                    ep, em = fd_energy(p0 + h * dt, w0), fd_energy(p0 - h * dt, w0)
                else:
                    ep, em = fd_energy(p0, w0 + h * dt), fd_energy(p0, w0 - h * dt)
                fd = (ep.item() - em.item()) / (2 * h)
                an = float(np.dot(g, d))
                worst = max(worst, abs(fd - an) / max(abs(fd), abs(an), 1e-12))
            assert worst <= 1e-6, (arg, worst)


def test_rrule_blocksparse_matches_oracle(nd):
    from oracle import blocksparse as obs
    A, B, _ = networks.qn_pair(512, seed=41)
    la, lb = (1, 2, -1), (-1, 3, 4)
    y, pb = nd.contract_rrule(nd.BlockSparseTensor.from_oracle(A), la, nd.BlockSparseTensor.from_oracle(B), lb)
    R, _ = obs.contract(A, la, B, lb)
    assert odense.rel_frobenius_error(y.data_numpy(), R.data) <= 1e-13
    import torch
    rng = np.random.default_rng(42)
    ybar = torch.from_numpy(rng.standard_normal(R.nnz)).cuda()
    Ab, Bb = pb(ybar)
    gA, gB = contract_pullback(A.to_dense(), (1, 2, 5), B.to_dense(), (5, 3, 4), (1, 2, 3, 4),
                               obs.BlockSparseTensor(R.inds, R.blocks, R.offsets, ybar.cpu().numpy()).to_dense())
    Ad = obs.BlockSparseTensor(A.inds, A.blocks, A.offsets, Ab.data_numpy()).to_dense()
    Bd = obs.BlockSparseTensor(B.inds, B.blocks, B.offsets, Bb.data_numpy()).to_dense()
    assert odense.rel_frobenius_error(Ad, gA) <= 1e-13
    assert odense.rel_frobenius_error(Bd, gB) <= 1e-13


def test_graph_captured_matvec(nd):
    """The four H_eff contractions captured once into a CUDA graph and replayed."""
    import ctypes as C
    import torch
    from ndtensors_gb300 import workloads as wl
    net = wl.qn_heff(chi=512, seed=5)
    G = {k: nd.BlockSparseTensor.from_host(net[k]) for k in ("L", "psi", "W1", "W2", "R")}
    steps = wl.heff_steps()
    rhs = [G["psi"], G["W1"], G["W2"], G["R"]]
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        cur, plans, outs = G["L"], [], []
        for (a, b, c), T in zip(steps, rhs):
            p = nd.get_plan(cur, a, T, b, c)
            o = nd.BlockSparseTensor(list(p.indsR), list(p.blocksR), list(p.offsetsR),
                                     torch.zeros(p.nnzR, dtype=torch.float64, device="cuda"))
            plans.append(p); outs.append(o); cur = o

        def run():
            x = G["L"]
            for (a, b, c), T, p, o in zip(steps, rhs, plans, outs):
                nd.contract_blocksparse(x, a, T, b, c, precision="ozaki", plan=p, out=o)
                x = o
        run()                                            # builds every per-plan cache outside capture
        torch.cuda.synchronize()
        eager = outs[-1].data.clone()
        outs[-1].data.zero_()
        h = nd.handle(0)
        h.call("nd_graph_begin")
        run()
        ge = C.c_void_p()
        h.call("nd_graph_end", C.byref(ge))
        for _ in range(2):
            outs[-1].data.zero_()
            h.call("nd_graph_launch", ge)
            torch.cuda.synchronize()
            assert torch.equal(outs[-1].data, eager)
        h.lib.nd_graph_destroy(ge)
