"""GB300 (sm_103a) implementation of Tichi_SPH's per-substep SPH hot path.

Public surface, named after the reference's modules:

* :mod:`.sph_config` -- ``Config`` from the reference's config / scenario JSON;
* :mod:`.sph_obj` -- ``Fluid`` particle sets (PyTorch CUDA tensors), ``Ngrid``,
  ``GlobalVariable``;
* :mod:`.sph` -- ``Solver`` (the CUDA context), ``cfl_condition``, ``sph_step``;
* :mod:`.simulation` -- the headless ``main.py``: scenario, ``run_step``, output.

The compute path is the C ABI of ``include/tichi_sph.h`` (``_lib/libtichi_sph.so``);
there is no CPU or Python fallback.
"""
from . import sph_config  # noqa: F401
from .sph_config import Config, load, from_argv  # noqa: F401
from .sph_obj import Fluid, Grid, Ngrid, GlobalVariable  # noqa: F401
from .sph import Solver, cfl_condition, map_velocity, sph_step  # noqa: F401
from .simulation import Simulation  # noqa: F401

__version__ = "0.1.0"
