"""GB300-native dual-particle SPH pressure projection (skytang0205/sand-water-coupling).

``DualParticleSphLiquid`` mirrors the reference's Simulation API over the C ABI
in include/swc.h, ``DEMParticleSand`` the DEM sand solver over include/swc_sand.h;
``Simulator`` drives either frame by frame as the reference's Simulator does;
``scenes`` builds the seeded synthetic workloads.
"""
from . import scenes  # noqa: F401
from ._lib import SwcError, load  # noqa: F401
from .liquid import DualParticleSphLiquid  # noqa: F401
from .sand import DEMParticleSand  # noqa: F401
from .simulator import Simulator  # noqa: F401

__all__ = ["DEMParticleSand", "DualParticleSphLiquid", "Simulator", "SwcError", "load", "scenes"]
