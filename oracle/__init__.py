"""CPU oracle of the reference renderer — test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU arms as the
checker; never by the svox2_gb300 package.
"""
