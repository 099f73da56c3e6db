"""diffsims_gb300 -- GB300-native (sm_103a) kinematical electron-diffraction
spot patterns, a drop-in for diffsims' ``SimulationGenerator.calculate_diffraction2d``
and ``get_kinematical_intensities``.

The compute path is the CUDA library ``libdiffsims_gb300.so`` (C ABI in
``include/diffsims_gb300.h``); there is no CPU fallback.
"""
from .crystal import Atom, Lattice, Phase, Rotation, Structure
from .generator import SimulationGenerator
from .sim_utils import get_electron_wavelength, get_kinematical_intensities
from .simulation2d import DiffractingVector, Simulation2D

__all__ = [
    "Atom", "Lattice", "Phase", "Rotation", "Structure", "SimulationGenerator", "Simulation2D",
    "DiffractingVector", "get_electron_wavelength", "get_kinematical_intensities",
]
__version__ = "0.1.0"
