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
    rotating z-x-z); ``struct_lib`` maps each identifier to that pair."""

    def __init__(self, identifiers, structures, orientations):
        for what, seq in (("structures", structures), ("orientations", orientations)):
            if len(seq) != len(identifiers):
                raise ValueError(f"Number of identifiers ({len(identifiers)}) and {what} ({len(seq)}) "
                                 f"must be the same.")
        self.identifiers = identifiers
        self.structures = structures
        self.orientations = orientations
        self.struct_lib = dict(zip(identifiers, zip(structures, orientations)))

    @classmethod
    def from_orientation_lists(cls, identifiers, structures, orientations):
        return cls(identifiers, structures, orientations)

    def get_library_size(self, to_print=False):
        """Number of orientations over all phases."""
        if to_print:
            for ident, ori in zip(self.identifiers, self.orientations):
                print(ident, "has", len(ori), "number of entries.")
        return int(sum(len(ori) for ori in self.orientations))


def load_DiffractionLibrary(filename, safety=False):
    """Load a pickled library; ``safety`` must acknowledge that unpickling
    runs code from the file."""
    if not safety:
        raise RuntimeError("Unpickling is risky, turn safety to True if you trust the author of this content")
    with open(filename, "rb") as handle:
        return pickle.load(handle)


def _get_library_entry_from_angles(library, phase, angles):
    """Index of the first orientation of ``phase`` whose Euler triple is
    within 1e-2 of ``angles`` (sum of absolute differences, degrees)."""
    table = np.asarray(library[phase]["orientations"], dtype=np.float64).reshape(-1, 3)
    hits = np.flatnonzero(np.abs(table - np.asarray(angles, dtype=np.float64)).sum(axis=1) < 1e-2)
    if hits.size == 0:
        raise ValueError("It appears that no library entry lies with 1e-2 of the target angle")
    return int(hits[0])


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
        """The simulation, intensities, pixel coordinates and intensity norm
        of one entry: the orientation nearest ``angle`` of ``phase``, or the
        first orientation of ``phase`` (of the first phase when none is
        given; an ``angle`` needs a ``phase``)."""
        if phase is None and angle is not None:
            raise ValueError("To select a certain angle you must first specify a phase")
        entry = self[phase] if phase is not None else next(iter(self.values()))
        k = _get_library_entry_from_angles(self, phase, angle) if angle is not None else 0
        inten = entry["intensities"][k]
        return {"Sim": entry["simulations"][k], "intensities": inten, "pixel_coords": entry["pixel_coords"][k],
                "pattern_norm": np.linalg.norm(inten)}

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
