"""CHECKER INFRASTRUCTURE: CPU oracle of the Disco RK substep cycle.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this package; the product never imports it."""
