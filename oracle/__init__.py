"""CPU oracle for the HT reduction -- test infrastructure only (see oracle.py)."""
