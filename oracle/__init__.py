"""CPU oracle for the Tree-SVD per-snapshot refresh.

TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; the product never imports it.
"""
