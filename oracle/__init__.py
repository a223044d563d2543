"""CPU oracle of the probe-particle AFM hot path -- test and benchmark infrastructure only.

Importable by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs; never by
the ppafm_gb300 package."""
