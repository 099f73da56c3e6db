"""``DiffractionSimulation``: the result container of the legacy
``DiffractionGenerator.calculate_ed_data``.

The interface is the one of diffsims/sims/diffraction_simulation.py:32-233
(names, arguments, the visible rows with and without the direct beam,
calibration, slicing, concatenation, in-plane rotate / shift) with the same
error types and messages.  The implementation is a view over one spot
table: the rows (x, y, z), Miller indices and intensities live in three
arrays of equal length, and every public accessor reads or writes the
*visible* rows -- all rows when the direct beam is kept, otherwise the rows
whose coordinates are not all zero.  Drawing (``get_diffraction_pattern``,
``get_as_mask``) is done by ``get_diffraction_pattern`` below on the GPU
rasteriser; ``plot`` (matplotlib) is not provided.
"""
from __future__ import annotations

import copy

import numpy as np


def _as_calibration(value):
    """None, or the per-axis calibration as a length-2 array (the reference's
    accepted forms and messages)."""
    if value is None:
        return None
    if np.all(np.equal(value, 0)):
        raise ValueError("`calibration` cannot be zero.")
    if isinstance(value, (float, int)):
        return np.full(2, float(value))
    if len(value) == 2:
        return np.asarray(value)
    raise ValueError("`calibration` must be a float or length-2tuple of floats.")


def _visible_column(column: str, doc: str):
    """A property reading / writing the visible rows of one spot-table column."""

    def get(self):
        return getattr(self, column)[self.direct_beam_mask]

    def put(self, value):
        getattr(self, column)[self.direct_beam_mask] = value

    return property(get, put, doc=doc)


class DiffractionSimulation:
    """Coordinates (n, 2 or 3, 1/Angstrom), Miller indices (n, 3) and
    intensities (n,) of one simulated pattern."""

    def __init__(self, coordinates, indices=None, intensities=None, calibration=None, offset=(0.0, 0.0),
                 with_direct_beam=False):
        xyz = np.atleast_2d(np.asarray(coordinates))
        n = xyz.shape[0]
        hkl = np.full((n, 3), np.nan) if indices is None else np.asarray(indices)
        inten = np.full(n, np.nan) if intensities is None else np.asarray(intensities)
        shapes_ok = xyz.ndim == 2 and hkl.ndim == 2 and inten.ndim == 1 and hkl.shape[0] == n == inten.shape[0]
        if not shapes_ok:
            raise ValueError("Coordinate, intensity, and indices lists must be of the correct and matching shape.")
        self._xyz, self._hkl, self._I = xyz, hkl, inten
        self.calibration = calibration
        self.offset = np.array(offset)
        self.with_direct_beam = with_direct_beam

    @classmethod
    def _from_arrays(cls, coordinates, indices, intensities, with_direct_beam):
        """A simulation from arrays already known to match (n, 3), (n, 3),
        (n,): the library's own results, without the constructor's checks."""
        obj = cls.__new__(cls)
        obj._xyz, obj._hkl, obj._I = coordinates, indices, intensities
        obj._calibration = None
        obj.offset = np.zeros(2)
        obj.with_direct_beam = with_direct_beam
        return obj

    # ---------------------------------------------------------- the table
    @property
    def direct_beam_mask(self):
        """Visible rows: all of them with the direct beam; otherwise the rows
        whose coordinates are not all zero."""
        if self.with_direct_beam:
            return np.ones(self._I.shape, dtype=bool)
        return self._xyz.any(axis=1)

    coordinates = _visible_column("_xyz", "Spot coordinates of the visible rows (1/Angstrom).")
    indices = _visible_column("_hkl", "Miller indices of the visible rows.")
    intensities = _visible_column("_I", "Intensities of the visible rows.")

    def __len__(self):
        return int(self.direct_beam_mask.sum())

    @property
    def size(self):
        return len(self)

    def __getitem__(self, sliced):
        xyz, hkl, inten = self.coordinates[sliced], self.indices[sliced], self.intensities[sliced]
        xyz, hkl, inten = np.atleast_2d(xyz), np.atleast_2d(hkl), np.atleast_1d(inten)
        if xyz.ndim != 2 or not 2 <= xyz.shape[1] <= 3:
            raise ValueError(f"Invalid slice: {sliced}")
        return DiffractionSimulation(xyz, indices=hkl, intensities=inten, calibration=self.calibration,
                                     offset=self.offset, with_direct_beam=self.with_direct_beam)

    def deepcopy(self):
        return copy.deepcopy(self)

    def __add__(self, other):
        out = self.deepcopy()
        out.extend(other)
        return out

    def extend(self, other):
        """Append another simulation's rows (all three columns; the
        reference stores the joined intensities under an unused name,
        diffraction_simulation.py:124-131, so its sum cannot be indexed)."""
        self._xyz = np.vstack([self._xyz, other._xyz])
        self._hkl = np.vstack([self._hkl, other._hkl])
        self._I = np.concatenate([self._I, other._I])

    # ------------------------------------------------------- calibration
    @property
    def calibration(self):
        return self._calibration

    @calibration.setter
    def calibration(self, value):
        self._calibration = _as_calibration(value)

    @property
    def calibrated_coordinates(self):
        """Coordinates in pixels: (xy + offset) / calibration."""
        if self.calibration is None:
            raise Exception("Pixel calibration is not set!")
        return (self.coordinates[:, :2] + self.offset) / self.calibration

    # ------------------------------------------------- in-plane transforms
    def _get_transformed_coordinates(self, angle, center=(0, 0), mirrored=False, units="real"):
        """The visible coordinates (``units``: 'real' or calibrated pixels)
        mirrored across x (optional), turned by ``angle`` degrees about the
        origin and shifted by ``center``: x + iy -> conj? * e^{i angle} + c
        (diffraction_simulation.py:199-215)."""
        out = (self.coordinates if units == "real" else self.calibrated_coordinates).astype(np.float64, copy=True)
        w = out[:, 0] + 1j * (-out[:, 1] if mirrored else out[:, 1])
        w = w * np.exp(1j * np.deg2rad(angle)) + complex(center[0], center[1])
        out[:, 0], out[:, 1] = w.real, w.imag
        return out

    def rotate_shift_coordinates(self, angle, center=(0, 0), mirrored=False):
        """In-plane rotation (degrees), mirror across x and shift, in place."""
        self.coordinates = self._get_transformed_coordinates(angle, center, mirrored, units="real")

    # ------------------------------------------------------------ drawing
    def get_diffraction_pattern(self, shape=(512, 512), sigma=10, direct_beam_position=None, in_plane_angle=0,
                                mirrored=False):
        """Detector image (float64 array of ``shape``) of this pattern, drawn
        by the GPU rasteriser: the calibrated spot positions turned by
        ``in_plane_angle`` (mirrored on request) about ``direct_beam_position``
        (default: the centre pixel), the spots in the frame truncated to
        whole pixels (last write wins), a Gaussian filter of ``sigma`` px
        (mode reflect), divided by the maximum; all zeros when no spot is in
        the frame (diffsims/sims/diffraction_simulation.py:296-354).  Needs
        the calibration."""
        from .engine import PhaseSpots, RasterSettings, rasterize
        if direct_beam_position is None:
            direct_beam_position = (shape[1] // 2, shape[0] // 2)
        pos = self._get_transformed_coordinates(in_plane_angle, direct_beam_position, mirrored, units="pixel")
        in_frame = (pos[:, 0] >= 0) & (pos[:, 0] < shape[1]) & (pos[:, 1] >= 0) & (pos[:, 1] < shape[0])
        if not in_frame.any():
            return np.zeros(shape)
        # pixel positions as they are: calibration 1, no turn, origin at (0, 0)
        rows = _Rows(np.c_[pos[:, :2], np.zeros(len(pos))], self.intensities)
        rs = RasterSettings(tuple(shape), sigma=sigma, calibration=1.0, direct_beam_position=(0.0, 0.0))
        return rasterize(PhaseSpots.from_vectors([rows]), rs)[0].cpu().numpy().astype(np.float64)

    def get_as_mask(self, shape, radius=6.0, negative=True, radius_function=None, direct_beam_position=None,
                    in_plane_angle=0, mirrored=False, *args, **kwargs):
        """Boolean image of discs of ``radius`` px (or ``radius_function(
        intensities)``) about the spots (diffsims/sims/diffraction_simulation.py:296-346);
        ``negative`` leaves the discs False on a True background."""
        r = radius_function(self.intensities, *args, **kwargs) if radius_function is not None else radius
        r = np.broadcast_to(np.asarray(r, dtype=np.float64), self.intensities.shape)
        if direct_beam_position is None:
            direct_beam_position = (shape[1] // 2, shape[0] // 2)
        pos = self._get_transformed_coordinates(in_plane_angle, direct_beam_position, mirrored, units="pixel")
        yy, xx = np.indices(shape)
        mask = np.zeros(shape, dtype=bool)
        for (x, y), rr in zip(pos[:, :2], r):
            mask |= (xx - x) ** 2 + (yy - y) ** 2 < rr ** 2
        return ~mask if negative else mask


class _Rows:
    """Spot rows in the form ``PhaseSpots.from_vectors`` takes."""

    def __init__(self, data, intensity):
        self.data, self.intensity, self.hkl = data, intensity, None


class ProfileSimulation:
    """A 1-D diffraction profile: peak magnitudes |g| (1/Angstrom),
    intensities (largest 100) and hkl labels (diffsims/sims/diffraction_simulation.py:460-480;
    ``get_plot`` is not provided)."""

    def __init__(self, magnitudes, intensities, hkls):
        self.magnitudes = magnitudes
        self.intensities = intensities
        self.hkls = hkls
