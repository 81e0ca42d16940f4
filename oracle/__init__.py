"""CPU oracle of BLAST's hot-path arithmetic (test infrastructure; see oracle.py)."""
