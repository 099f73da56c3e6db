"""``Simulation1D``: the 1-D profile returned by
``SimulationGenerator.calculate_diffraction1d``.

Mirrors diffsims/simulations/simulation1d.py:30-75 (attributes, ``repr``,
``theta``); ``plot`` (matplotlib) is not provided.
"""
from __future__ import annotations

import numpy as np


class Simulation1D:
    """Peak spacings |g| (1/Angstrom), intensities (largest 100) and indices
    (hkl, or hkil for hexagonal lattices) of one phase."""

    def __init__(self, phase, reciprocal_spacing, intensities, hkl, reciprocal_radius, wavelength):
        self.phase = phase
        self.reciprocal_spacing = reciprocal_spacing
        self.intensities = intensities
        self.hkl = hkl
        self.reciprocal_radius = reciprocal_radius
        self.wavelength = wavelength

    def __repr__(self):
        return f"Simulation1D(name: {self.phase.name}, wavelength: {self.wavelength})"

    @property
    def theta(self):
        """Scattering angles arctan(|g| / k0) (radians)."""
        return np.arctan2(np.array(self.reciprocal_spacing), 1 / self.wavelength)
