"""CPU oracle for the GB300 backend's parity tests.

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
legs may use this package as the checker.  The product package (opensbli_gb300) never imports it.
"""
