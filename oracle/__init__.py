"""ORACLE -- test infrastructure only.

CPU restatements of the reference's slicing / matching / merge path, used by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.
Nothing in spinifel_gb300/ imports this package.
"""
