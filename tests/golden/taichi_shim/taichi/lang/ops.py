"""``taichi.lang.ops`` names the reference imports; rewritten away inside kernels."""
from taichi import atomic_add, atomic_min, atomic_max, sqrt  # noqa: F401
