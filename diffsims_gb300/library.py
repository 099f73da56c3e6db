"""Template libraries of the legacy path: ``StructureLibrary``,
``DiffractionLibrary`` and ``DiffractionLibraryGenerator``.

Mirrors diffsims/libraries/structure_library.py:24-110,
diffsims/libraries/diffraction_library.py:29-180 and
``DiffractionLibraryGenerator.get_diffraction_library``
(diffsims/generators/library_generator.py:36-155): same names, arguments,
entries and errors.  The reference calls ``calculate_ed_data`` once per
orientation in a Python loop; here every orientation of a phase is one GPU
launch (``DiffractionGenerator.calculate_ed_data`` with an (N, 3) array of
Euler angles).
"""
from __future__ import annotations

import pickle

import numpy as np


class StructureLibrary:
    """Phase identifiers -> (structure, list of Euler triples in degrees,
    rotating z-x-z)."""

    def __init__(self, identifiers, structures, orientations):
        if len(identifiers) != len(structures):
            raise ValueError("Number of identifiers ({}) and structures ({}) must be the same.".format(
                len(identifiers), len(structures)))
        if len(identifiers) != len(orientations):
            raise ValueError("Number of identifiers ({}) and orientations ({}) must be the same.".format(
                len(identifiers), len(orientations)))
        self.identifiers = identifiers
        self.structures = structures
        self.orientations = orientations
        self.struct_lib = dict()
        for ident, struct, ori in zip(identifiers, structures, orientations):
            self.struct_lib[ident] = (struct, ori)

    @classmethod
    def from_orientation_lists(cls, identifiers, structures, orientations):
        return cls(identifiers, structures, orientations)

    def get_library_size(self, to_print=False):
        """Total number of orientations (a one-entry list counts as one)."""
        size_library = 0
        for i in range(len(self.orientations)):
            size_library += 1 if len(self.orientations[i]) == 1 else len(self.orientations[i])
            if to_print:
                print(self.identifiers[i], "has", len(self.orientations[i]), "number of entries.")
        return size_library


def load_DiffractionLibrary(filename, safety=False):
    """Load a pickled library; ``safety`` must acknowledge that unpickling
    runs code from the file."""
    if safety:
        with open(filename, "rb") as handle:
            return pickle.load(handle)
    raise RuntimeError("Unpickling is risky, turn safety to True if you trust the author of this content")


def _get_library_entry_from_angles(library, phase, angles):
    """Index of the first orientation within 1e-2 (sum of absolute angle
    differences, degrees) of ``angles``."""
    for orientation_index, orientation in enumerate(library[phase]["orientations"]):
        if np.sum(np.abs(np.subtract(orientation, angles))) < 1e-2:
            return orientation_index
    raise ValueError("It appears that no library entry lies with 1e-2 of the target angle")


class DiffractionLibrary(dict):
    """Phase identifier -> {"simulations", "orientations", "pixel_coords",
    "intensities"}, with the generating settings as attributes."""

    def __init__(self, *args, **kwargs):
        super().__init__(*args, **kwargs)
        self.identifiers = None
        self.structures = None
        self.diffraction_generator = None
        self.reciprocal_radius = 0.0
        self.with_direct_beam = False

    def get_library_entry(self, phase=None, angle=None):
        if phase is not None:
            phase_entry = self[phase]
            orientation_index = _get_library_entry_from_angles(self, phase, angle) if angle is not None else 0
        elif angle is not None:
            raise ValueError("To select a certain angle you must first specify a phase")
        else:
            phase_entry = next(iter(self.values()))
            orientation_index = 0
        return {
            "Sim": phase_entry["simulations"][orientation_index],
            "intensities": phase_entry["intensities"][orientation_index],
            "pixel_coords": phase_entry["pixel_coords"][orientation_index],
            "pattern_norm": np.linalg.norm(phase_entry["intensities"][orientation_index]),
        }

    def pickle_library(self, filename):
        with open(filename, "wb") as handle:
            pickle.dump(self, handle, protocol=pickle.HIGHEST_PROTOCOL)


class DiffractionLibraryGenerator:
    """Simulations of every (phase, orientation) of a ``StructureLibrary``
    with a ``DiffractionGenerator``."""

    def __init__(self, electron_diffraction_calculator):
        self.electron_diffraction_calculator = electron_diffraction_calculator

    def get_diffraction_library(self, structure_library, calibration, reciprocal_radius, half_shape,
                                with_direct_beam=True, max_excitation_error=1e-2, shape_factor_width=None,
                                debye_waller_factors={}):
        """library_generator.py:51-155: per phase, the simulations of all its
        orientations (one launch), their pixel coordinates
        ``rint(calibrated xy + half_shape)`` and intensities."""
        library = DiffractionLibrary()
        diffractor = self.electron_diffraction_calculator
        if shape_factor_width is None:
            shape_factor_width = max_excitation_error
        for phase_name in structure_library.struct_lib.keys():
            structure, orientations = structure_library.struct_lib[phase_name]
            n = len(orientations)
            simulations = np.empty(n, dtype="object")
            pixel_coords = np.empty(n, dtype="object")
            intensities = np.empty(n, dtype="object")
            if n:
                sims = diffractor.calculate_ed_data(
                    structure, reciprocal_radius, rotation=np.asarray(orientations, dtype=np.float64).reshape(-1, 3),
                    with_direct_beam=with_direct_beam, max_excitation_error=max_excitation_error,
                    shape_factor_width=shape_factor_width, debye_waller_factors=debye_waller_factors)
                for i, simulation in enumerate(sims):
                    simulation.calibration = calibration
                    simulations[i] = simulation
                    pixel_coords[i] = np.rint(simulation.calibrated_coordinates[:, :2] + half_shape).astype(int)
                    intensities[i] = simulation.intensities
            library[phase_name] = {"simulations": simulations, "orientations": orientations,
                                   "pixel_coords": pixel_coords, "intensities": intensities}
        library.identifiers = structure_library.identifiers
        library.structures = structure_library.structures
        library.diffraction_generator = diffractor
        library.reciprocal_radius = reciprocal_radius
        library.with_direct_beam = with_direct_beam
        return library
