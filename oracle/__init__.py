"""CPU oracle of the GI path: test infrastructure only (see oracle.py)."""
