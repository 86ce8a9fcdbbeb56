"""CPU oracle of the SODA path — test infrastructure only (see oracle.py)."""
