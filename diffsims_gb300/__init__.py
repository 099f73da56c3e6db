"""diffsims_gb300 -- GB300-native (sm_103a) kinematical electron-diffraction
spot patterns, a drop-in for diffsims' ``SimulationGenerator.calculate_diffraction2d``
and ``get_kinematical_intensities``, with the 1-D profiles, the legacy
``DiffractionGenerator`` and template libraries, and the structure-factor
helpers (``diffsims_gb300.structure_factor``) on the same kernels.

The compute path is the CUDA library ``libdiffsims_gb300.so`` (C ABI in
``include/diffsims_gb300.h``); there is no CPU fallback.
"""
from .crystal import Atom, Lattice, Phase, Rotation, Structure
from .diffraction_generator import DiffractionGenerator
from .diffraction_simulation import DiffractionSimulation, ProfileSimulation
from .generator import SimulationGenerator
from .library import DiffractionLibrary, DiffractionLibraryGenerator, StructureLibrary
from .sim_utils import get_electron_wavelength, get_kinematical_intensities
from .simulation1d import Simulation1D
from .simulation2d import DiffractingVector, Simulation2D

__all__ = [
    "Atom", "Lattice", "Phase", "Rotation", "Structure", "SimulationGenerator", "Simulation1D", "Simulation2D",
    "DiffractingVector", "get_electron_wavelength", "get_kinematical_intensities", "DiffractionGenerator",
    "DiffractionSimulation", "ProfileSimulation", "DiffractionLibrary", "DiffractionLibraryGenerator",
    "StructureLibrary",
]
__version__ = "0.1.0"
