"""ORACLE — test infrastructure only: CPU restatement of the reference algorithm.

Only tests/, __graft_entry__.smoke() and the CPU-baseline legs of bench.py may use this package.
"""
