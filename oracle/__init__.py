"""CPU oracle for the gCQ queues: test infrastructure, not the product.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline and reference arm
may use this package, and only as the checker or the timed CPU baseline.  Parity is pinned here:
the linearizability checker accepts both histories the reference ships
(correctness/histories/*.jsonl) and rejects the mutated copies of them.
"""
