"""ORACLE - test infrastructure only.

CPU restatements of PyCD's Ewald array and KMC loop, pinned against the
reference's golden vectors under tests/golden.  Only tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline / reference legs use
this package, and only as the checker or the timed CPU baseline.  The
product package (pycd_gb300) never imports it.
"""
