"""CPU oracle of the stloufra/LB solver path.  TEST INFRASTRUCTURE ONLY: imported by tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg, never by the product package."""
