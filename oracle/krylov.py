"""Lanczos basis construction (oracle restatement, CPU, numpy) -- test infrastructure.

The local eigenproblem of a DMRG sweep is solved by KrylovKit, called from
ITensorMPS (neither is part of the reference repository).  The reference supplies
the vector-space interface KrylovKit consumes, ITensorsVectorInterfaceExt
(ext/ITensorsVectorInterfaceExt/ITensorsVectorInterfaceExt.jl:5-84;
`[compat] VectorInterface = "0.4, 0.5"`, Project.toml:69).  KrylovKit's Lanczos
follows the published recurrence (Lanczos 1950) with re-orthogonalisation of each
new vector against the basis.  This restatement uses classical
Gram-Schmidt applied twice against the whole basis, the form the device solver
implements: for j = 0 .. k-1
    w = H v_j;  c = V_j^T w;  w -= V_j c;  c' = V_j^T w;  w -= V_j c'
    alpha_j = c_j + c'_j;  beta_j = |w|;  v_{j+1} = w / beta_j
and the Ritz pair of the tridiagonal T = tridiag(beta, alpha, beta).
"""
import numpy as np


def lanczos(apply, v0, krylovdim):
    n = v0.size
    V = np.zeros((krylovdim + 1, n))
    alpha = np.zeros(krylovdim)
    beta = np.zeros(krylovdim)
    V[0] = v0 / np.linalg.norm(v0)
    for j in range(krylovdim):
        w = apply(V[j])
        c = V[:j + 1] @ w
        w = w - V[:j + 1].T @ c
        c2 = V[:j + 1] @ w
        w = w - V[:j + 1].T @ c2
        alpha[j] = c[j] + c2[j]
        beta[j] = np.linalg.norm(w)
        V[j + 1] = w / beta[j]
    T = np.diag(alpha) + np.diag(beta[:-1], 1) + np.diag(beta[:-1], -1)
    vals, vecs = np.linalg.eigh(T)
    return vals[0], V[:krylovdim].T @ vecs[:, 0], alpha, beta
