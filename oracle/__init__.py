"""CPU oracle of the hot path (test infrastructure; see oracle/oracle.py)."""
