"""CPU oracle for foeuler's implicit inner loop -- TEST INFRASTRUCTURE ONLY.

A plain-C restatement of the reference arithmetic (fos_oracle.c) and its ctypes
binding (pyoracle.py).  Used by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg, to check results and time the CPU path; the fosolvers_gb300 package
never imports it.
"""
