"""ORACLE -- test infrastructure only (never imported by the camb_gb300 package).

CPU restatement of the reference's scalar flat hot path (camb_oracle.cpp), used by
tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg as the checker.
"""
