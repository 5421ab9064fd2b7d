"""GB300 global-placement core: a drop-in for RePlAce's initial place and
Nesterov loop, computed by hand-written sm_103a kernels behind a C ABI
(include/gpl.h, libgpl_gb300.so)."""

from . import lefdef, netlist  # noqa: F401
from ._abi import default_params  # noqa: F401
from ._lib import GplError, load  # noqa: F401
from .placer import (Placer, Replace, batch_initial_place, batch_nesterov_run, global_placement,  # noqa: F401
                     poisson_solve)
from .server import PlacementServer  # noqa: F401

__all__ = ["Placer", "Replace", "batch_initial_place", "batch_nesterov_run", "global_placement", "poisson_solve",
           "GplError", "load", "default_params", "lefdef", "netlist", "PlacementServer"]
