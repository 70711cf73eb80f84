"""CPU oracle for the GB300 kernels — TEST INFRASTRUCTURE ONLY.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg; the lofloat_gb300 package never imports it.
"""
