"""CPU oracle of the minimc particle-history path.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() (as the
checker) and bench.py's CPU-baseline leg.  The GPU engine never uses it.
"""
