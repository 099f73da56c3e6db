"""``DiffractionSimulation``: the result container of the legacy
``DiffractionGenerator.calculate_ed_data``.

Mirrors diffsims/sims/diffraction_simulation.py:32-233 (constructor checks,
the direct-beam mask, calibration and offset, slicing, concatenation and the
in-plane rotate / shift of the coordinates) with the same names and errors.
Its drawing methods (``get_diffraction_pattern``, ``get_as_mask``, ``plot``:
numba, PIL and matplotlib in the reference) are not provided; detector
images of the current path come from ``Simulation2D`` and the GPU rasteriser.
"""
from __future__ import annotations

import copy

import numpy as np


class DiffractionSimulation:
    """Coordinates (n, 2 or 3, 1/Angstrom), Miller indices (n, 3) and
    intensities (n,) of one simulated pattern."""

    def __init__(self, coordinates, indices=None, intensities=None, calibration=None, offset=(0.0, 0.0),
                 with_direct_beam=False):
        coordinates = np.asarray(coordinates)
        if coordinates.ndim == 1:
            coordinates = coordinates[None, :]
        if indices is None:
            indices = np.full((coordinates.shape[0], 3), np.nan)
        if intensities is None:
            intensities = np.full((coordinates.shape[0]), np.nan)
        indices, intensities = np.asarray(indices), np.asarray(intensities)
        if (coordinates.shape[0] == indices.shape[0] == intensities.shape[0]
                and coordinates.ndim == indices.ndim == 2 and intensities.ndim == 1):
            self._coordinates = coordinates
            self._indices = indices
            self._intensities = intensities
        else:
            raise ValueError("Coordinate, intensity, and indices lists must be of the correct and matching shape.")
        self.calibration = calibration
        self.offset = np.array(offset)
        self.with_direct_beam = with_direct_beam

    @classmethod
    def _from_arrays(cls, coordinates, indices, intensities, with_direct_beam):
        """A simulation from arrays already known to match (n, 3), (n, 3),
        (n,): the library's own results, without the constructor's checks."""
        obj = cls.__new__(cls)
        obj._coordinates, obj._indices, obj._intensities = coordinates, indices, intensities
        obj._calibration = None
        obj.offset = np.zeros(2)
        obj.with_direct_beam = with_direct_beam
        return obj

    def __len__(self):
        return self.coordinates.shape[0]

    @property
    def size(self):
        return self.__len__()

    def __getitem__(self, sliced):
        coords = self.coordinates[sliced]
        inds = self.indices[sliced]
        ints = self.intensities[sliced]
        if coords.ndim == 1:
            coords, inds, ints = coords[None, :], inds[None, :], ints[None]
        if coords.ndim > 2 or coords.shape[1] > 3 or coords.shape[1] < 2:
            raise ValueError(f"Invalid slice: {sliced}")
        return DiffractionSimulation(coords, indices=inds, intensities=ints, calibration=self.calibration,
                                     offset=self.offset, with_direct_beam=self.with_direct_beam)

    def deepcopy(self):
        return copy.deepcopy(self)

    def __add__(self, other):
        new = self.deepcopy()
        new.extend(other)
        return new

    def extend(self, other):
        """Append the spots of another simulation.  The reference assigns the
        concatenated intensities to an unused attribute
        (diffraction_simulation.py:124-131), which leaves the arrays with
        different lengths; here they are appended."""
        self._coordinates = np.concatenate([self._coordinates, other._coordinates], axis=0)
        self._indices = np.concatenate([self._indices, other._indices], axis=0)
        self._intensities = np.concatenate([self._intensities, other._intensities], axis=0)

    @property
    def indices(self):
        return self._indices[self.direct_beam_mask]

    @indices.setter
    def indices(self, indices):
        self._indices[self.direct_beam_mask] = indices

    @property
    def calibrated_coordinates(self):
        """Coordinates in pixels: (xy + offset) / calibration."""
        if self.calibration is not None:
            return (self.coordinates[:, :2] + self.offset) / self.calibration
        raise Exception("Pixel calibration is not set!")

    @property
    def calibration(self):
        return self._calibration

    @calibration.setter
    def calibration(self, calibration):
        if calibration is None:
            pass
        elif np.all(np.equal(calibration, 0)):
            raise ValueError("`calibration` cannot be zero.")
        elif isinstance(calibration, (float, int)):
            calibration = np.array((calibration, calibration))
        elif len(calibration) == 2:
            calibration = np.array(calibration)
        else:
            raise ValueError("`calibration` must be a float or length-2tuple of floats.")
        self._calibration = calibration

    @property
    def direct_beam_mask(self):
        """All True with the direct beam; else False where every coordinate is 0."""
        if self.with_direct_beam:
            return np.ones_like(self._intensities, dtype=bool)
        return np.any(self._coordinates, axis=1)

    @property
    def coordinates(self):
        return self._coordinates[self.direct_beam_mask]

    @coordinates.setter
    def coordinates(self, coordinates):
        self._coordinates[self.direct_beam_mask] = coordinates

    @property
    def intensities(self):
        return self._intensities[self.direct_beam_mask]

    @intensities.setter
    def intensities(self, intensities):
        self._intensities[self.direct_beam_mask] = intensities

    def _get_transformed_coordinates(self, angle, center=(0, 0), mirrored=False, units="real"):
        """Rotate by ``angle`` degrees (optionally mirrored across x) and shift
        (diffraction_simulation.py:199-215)."""
        coords = self.coordinates.copy() if units == "real" else self.calibrated_coordinates.copy()
        cx, cy = center
        x, y = coords[:, 0], coords[:, 1]
        theta = (-1 if mirrored else 1) * np.arctan2(y, x) + np.deg2rad(angle)
        rd = np.sqrt(x ** 2 + y ** 2)
        coords[:, 0] = rd * np.cos(theta) + cx
        coords[:, 1] = rd * np.sin(theta) + cy
        return coords

    def rotate_shift_coordinates(self, angle, center=(0, 0), mirrored=False):
        """In-plane rotation (degrees), mirror across x and shift, in place."""
        self.coordinates = self._get_transformed_coordinates(angle, center, mirrored, units="real")


class ProfileSimulation:
    """A 1-D diffraction profile: peak magnitudes |g| (1/Angstrom),
    intensities (largest 100) and hkl labels (diffsims/sims/diffraction_simulation.py:460-480;
    ``get_plot`` is not provided)."""

    def __init__(self, magnitudes, intensities, hkls):
        self.magnitudes = magnitudes
        self.intensities = intensities
        self.hkls = hkls
