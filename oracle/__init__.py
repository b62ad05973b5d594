"""CPU oracle of the reference kernels: test infrastructure only (see oracle.py)."""
