"""Sub-package of the pure-Python Taichi stand-in (test infrastructure only)."""
