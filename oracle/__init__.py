"""CPU oracle for the monodomain time step - TEST INFRASTRUCTURE ONLY.

Only tests/, the smoke check in __graft_entry__.py and bench.py's CPU-baseline
leg import this package, and only as the checker.  See oracle.h for what each
part restates from the reference and how it is pinned.
"""
