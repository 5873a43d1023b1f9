"""CPU oracle for the x2dhf (MC)SOR relaxation path -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
reference arm) import this package.  The GPU product never does.
"""
