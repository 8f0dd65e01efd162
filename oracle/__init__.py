"""CPU oracle for the w-stacking hot path -- test infrastructure only.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg.  The product library (lofar_gb300) never imports it.
"""
