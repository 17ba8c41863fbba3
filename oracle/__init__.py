"""CPU oracle for the NDTensors contraction hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library imports, links or
calls this package.  It is a plain numpy restatement of the reference's CPU
algorithms (ITensors.jl / NDTensors.jl), used by ``tests/``, by
``__graft_entry__.smoke()`` and by ``bench.py``'s CPU-baseline leg as the
checker.  Every function cites the reference file:line it follows (paths are
relative to the ITensors.jl repository root).

Modules
-------
labels      ncon label logic (``compute_contraction_labels``, ``contract_labels``).
qn          U(1) QN index model, ``flux``, ``nzblocks``, combined-index blocks.
dense       dense ``contract!`` with alpha/beta, ``permutedims!`` with fused f.
blocksparse BlockSparse storage, sequential block plan (bit-exact structure),
            grouped block contraction, block permutedims, combiner matricization.
truncate    ``truncate!`` (exact restatement of the scalar loop).
linalg      blockwise ``svd`` / ``qr`` (LAPACK gesdd / geqrf via numpy).
networks    seeded synthetic workloads (dense pair, dense H_eff, QN pair,
            QN two-site H_eff, XXZ MPO).
adjoint     the contraction pullback (``rrule(contract)``).

Parity pinning: the reference ships no stored golden vectors for this path.
The oracle is pinned against the known-answer tests in the reference's own
test files (transcribed as JSON under ``tests/golden/``); values elsewhere are
pinned only to a dense numpy recomputation, as the reference's tests are.
"""
