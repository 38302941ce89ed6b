"""Parity oracle for the PBF fluid step: test infrastructure only.

The product package (novaphy_gb300) never imports this package; tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use it as the checker.
"""
