"""CPU oracle of the SPH hot path (a C restatement of the reference's src/ solver).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU
legs, as the checker.  The product never calls it.
"""
