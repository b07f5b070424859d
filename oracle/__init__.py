"""CPU oracle for the 2-site DMRG hot path of amiragha/mps (NumPy float64 restatement).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` as the checker.  The GPU library never imports, links or calls anything here.

Parity status: the SymTensors bookkeeping and contraction path are pinned by the reference's own
known-answer tests (test/symtensortests.jl, test/mpotests.jl), restated in
tests/test_oracle_kats.py.  The Krylov eigensolver boundary (KrylovKit, unvendored and unpinned)
is "parity unpinned".
"""
