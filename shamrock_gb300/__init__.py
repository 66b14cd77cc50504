"""GB300-native SPH timestep hot path for Shamrock's shammodels::sph solver.

The compute path is ``libgbsph.so`` (hand-written sm_103a CUDA behind the C ABI
declared in include/gbsph.h).  This package adds the reference-shaped Python
model interface (``get_Model_SPH``), module-level wrappers on torch tensors, the
synthetic workload generators and the differentiable step.
"""

from ._lib import GbsphError  # noqa: F401
from .model import Context, Model, SolverConfig, UnitSystem, get_Model_SPH  # noqa: F401
from .phantom import PhantomDump, compare_phantom_dumps, load_phantom_dump  # noqa: F401

__all__ = ["Context", "GbsphError", "Model", "SolverConfig", "UnitSystem", "get_Model_SPH",
           "PhantomDump", "compare_phantom_dumps", "load_phantom_dump"]
__version__ = "0.1.0"
