"""GB300-native batched stabilizer-tableau simulator.

Drop-in for the reference package ``plaquette_simulator``
(plaquette_simulator/__init__.py:2-4): ``plaquette_simulator.CliffordState``
runs every gate and measurement in hand-written sm_103a CUDA kernels.
"""
from .simulator import CliffordState
from . import circuits

__version__ = "0.1.0"

__all__ = ["CliffordState", "circuits", "__version__"]
