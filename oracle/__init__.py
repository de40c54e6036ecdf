"""FP64 CPU oracle for the KillingFusion hot path (TEST INFRASTRUCTURE ONLY).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs as
the checker; the product package never imports it.
"""
