"""Test oracle for the GB300 GPMA+ (CPU restatement + reference driver I/O).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.
"""
