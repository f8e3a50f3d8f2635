"""CPU oracle of the MGPBD step (test infrastructure only).

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
and only there, as the checker.  The product path (controllable_pbd_3d_gb300)
never imports it.
"""
