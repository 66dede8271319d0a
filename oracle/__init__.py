"""CPU oracle for the RandBLAS sketching hot path -- test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg; never by the
product package randblas_gb300.
"""
