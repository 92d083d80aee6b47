"""CPU restatement of ETHER's Monte Carlo sweep -- TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg, as the
checker.  The product (ether_gb300, libether_gpu.so) never imports or links it.
"""
