"""ORACLE -- test infrastructure, not product code.

CPU restatement of the reference DiskDyn hot path (ddx_oracle.c) and a runner for the
reference's own kernels compiled for sm_103a (ref/).  Only tests/, the smoke check of
__graft_entry__ and the CPU-baseline legs of bench.py use this package.
"""
