"""CPU oracle for the ASTC encoder (test infrastructure; see oracle.py)."""
