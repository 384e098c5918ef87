"""CPU oracle (test infrastructure): the parity checker and CPU baseline.

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
legs may import this package.  The product library never loads it.
"""
