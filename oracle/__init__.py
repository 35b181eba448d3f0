"""CPU FP64 oracle for the topomax elasticity design loop.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package (``topomax_gb300``)
imports this package; it is used by ``tests/``, by ``__graft_entry__.smoke()``
and by ``bench.py``'s CPU-baseline / reference arm as the checker.

Parity is pinned against the reference's known-answer test
``tests/test_elasticity_solver.py:30-55`` (triangle design, N=10, objective
0.0018191324070894702 at k=24) -- see ``tests/test_oracle.py``.
"""
