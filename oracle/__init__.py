"""CPU oracle of the renderer's hot path: test infrastructure only (see oracle.py)."""
