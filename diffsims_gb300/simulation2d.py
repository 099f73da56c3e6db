"""Result containers: ``Simulation2D`` and ``DiffractingVector``.

Mirror the parts of diffsims/simulations/simulation2d.py (``Simulation2D``,
:109-764) and diffsims/crystallography/_diffracting_vector.py
(``DiffractingVector``) that users of ``calculate_diffraction2d`` read: the
phase x rotation nesting, the ``iphase`` / ``irot`` selectors, the
phase / rotation cursor and iteration, per-pattern spot vectors with
``data`` / ``intensity`` / ``hkl``, in-plane transforms,
``polar_flatten_simulations`` and ``get_diffraction_pattern``.  Spots stay
on the device in CSR form until a pattern is accessed; plotting is not
provided.
"""
from __future__ import annotations

import copy

import numpy as np

from .crystal import Rotation


class DiffractingVector:
    """Spots of one pattern: beam-frame ``data`` (n, 3) in 1/Angstrom,
    ``intensity`` (n,), Miller indices ``hkl`` (n, 3)."""

    def __init__(self, phase, xyz, intensity=None, hkl=None, rotation=None):
        self.phase = phase
        self.data = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        n = self.data.shape[0]
        self._intensity = np.full(n, np.nan) if intensity is None else np.asarray(intensity, dtype=np.float64)
        if self._intensity.shape[0] != n:
            raise ValueError("Length of intensity array must match number of vectors")
        self._hkl = None if hkl is None else np.asarray(hkl, dtype=np.float64).reshape(-1, 3)
        self.rotation = rotation

    @property
    def size(self):
        return self.data.shape[0]

    @property
    def shape(self):
        return (self.size,)

    def __len__(self):
        return self.size

    @property
    def x(self):
        return self.data[:, 0]

    @property
    def y(self):
        return self.data[:, 1]

    @property
    def z(self):
        return self.data[:, 2]

    @property
    def intensity(self):
        return self._intensity

    @intensity.setter
    def intensity(self, value):
        if not hasattr(value, "__len__"):
            value = np.array([value] * self.size)
        if len(value) != self.size:
            raise ValueError("Length of intensity array must match number of vectors")
        self._intensity = np.array(value, dtype=np.float64)

    @property
    def hkl(self):
        return self._hkl

    @property
    def gspacing(self):
        return np.linalg.norm(self.data, axis=1)

    @property
    def dspacing(self):
        return 1.0 / self.gspacing

    def calculate_structure_factor(self):
        """Not available on spot vectors, as in the reference
        (diffsims/crystallography/_diffracting_vector.py:180-184): the
        intensities already hold |F|^2 times the shape factor."""
        raise NotImplementedError("Structure factor calculation not implemented for DiffractionVector. "
                                  "Use ReciprocalLatticeVector instead.")

    def __getitem__(self, key):
        if isinstance(key, (int, np.integer)):
            key = slice(key, key + 1 if key != -1 else None)
        return DiffractingVector(self.phase, self.data[key], self._intensity[key],
                                 None if self._hkl is None else self._hkl[key], self.rotation)

    def flatten(self):
        return self

    def to_flat_polar(self):
        """(r, theta) of the spots projected on the x, y plane
        (diffsims/crystallography/_diffracting_vector.py:186-194)."""
        r = np.linalg.norm(self.data[:, :2], axis=1)
        return r, np.arctan2(self.data[:, 1], self.data[:, 0])

    def __repr__(self):
        name = getattr(self.phase, "name", "")
        return f"DiffractingVector ({self.size},), {name}"


class _PhaseCoordinates:
    """Lazy sequence of one phase's patterns (CSR on the device)."""

    def __init__(self, phase, spots, rotation):
        self.phase = phase
        self.spots = spots
        self.rotation = rotation

    def __len__(self):
        return self.spots.n_orient

    @property
    def size(self):
        return len(self)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[k] for k in range(*i.indices(len(self)))]
        n = len(self)
        if i < 0:
            i += n
        if not 0 <= i < n:
            raise IndexError(i)
        hkl, xyz, inten = self.spots.pattern(i)
        return DiffractingVector(self.phase, xyz, inten, hkl, self.rotation[i])

    def __iter__(self):
        for i in range(len(self)):
            yield self[i]


class _PhaseSelector:
    """``Simulation2D.iphase[item]``: the phases ``item`` (a name, an index
    or a slice) as a new ``Simulation2D`` over the same device spots
    (diffsims/simulations/simulation2d.py:43-73)."""

    def __init__(self, sim):
        self.sim = sim

    def __getitem__(self, item):
        sim = self.sim
        if not sim._multi_phase:
            raise ValueError("Only one phase in the simulation")
        plist, rlist = list(sim.phases), list(sim.rotations)
        if isinstance(item, str):
            item = [getattr(p, "name", None) for p in plist].index(item)
        elif not isinstance(item, (int, np.integer, slice)):
            raise ValueError("Item must be a string or integer")
        # an index gives a one-phase simulation, a slice a list of phases
        return Simulation2D(plist[item], sim._spots[item], rlist[item], sim.simulation_generator,
                            sim.reciprocal_radius)


class _RotationSelector:
    """``Simulation2D.irot[item]``: the rotations ``item`` of every phase as
    a new ``Simulation2D`` (their spots gathered on the device;
    diffsims/simulations/simulation2d.py:76-106)."""

    def __init__(self, sim):
        self.sim = sim

    def __getitem__(self, item):
        sim = self.sim
        if sim.current_size == 1:
            raise ValueError("Only one rotation in the simulation")
        if not sim._multi_phase:
            return Simulation2D(sim.phases, sim._spots[0].select(item), sim.rotations[item],
                                sim.simulation_generator, sim.reciprocal_radius)
        return Simulation2D(sim.phases, [s.select(item) for s in sim._spots], [r[item] for r in sim.rotations],
                            sim.simulation_generator, sim.reciprocal_radius)


class Simulation2D:
    """Result of ``SimulationGenerator.calculate_diffraction2d``.

    ``phases``, ``rotations`` and ``coordinates`` nest as in the reference
    (diffsims/generators/simulation_generator.py:244-258): one phase and one
    rotation -> ``coordinates`` is a ``DiffractingVector``; one phase and N
    rotations -> a sequence of N; P phases -> a list of P sequences.
    """

    def __init__(self, phases, coordinates, rotations, simulation_generator, reciprocal_radius=1.0):
        """Same arguments as the reference (simulation2d.py:115-186).
        ``coordinates`` is what ``calculate_diffraction2d`` hands over (one
        ``PhaseSpots`` per phase, device CSR) or, as in the reference,
        ``DiffractingVector`` objects: one (single rotation), a sequence (one
        phase), or a list of sequences (several phases); these are uploaded
        into the same device CSR form."""
        from .engine import PhaseSpots
        self._multi_phase = isinstance(phases, (list, tuple, np.ndarray))
        plist = list(phases) if self._multi_phase else [phases]
        rlist = list(rotations) if self._multi_phase else [rotations]
        if len(rlist) != len(plist):
            raise ValueError(f"The number of rotations: {len(rlist)} must match the number of phases {len(plist)}")
        if isinstance(coordinates, PhaseSpots):
            spots = [coordinates]
        elif (isinstance(coordinates, (list, tuple)) and coordinates
              and all(isinstance(c, PhaseSpots) for c in coordinates)):
            spots = list(coordinates)
        else:
            clist = list(coordinates) if self._multi_phase else [coordinates]
            if len(clist) != len(plist):
                raise ValueError(f"{len(clist)} coordinate sets for {len(plist)} phases")
            spots = []
            for c, r in zip(clist, rlist):
                vecs = [c] if isinstance(c, DiffractingVector) else list(c)
                n_rot = getattr(r, "size", 1)
                if n_rot != len(vecs):
                    raise ValueError(f"The number of rotations: {n_rot} must match the number of "
                                     f"coordinates {len(vecs)}")
                spots.append(PhaseSpots.from_vectors(vecs))
        self.phases = phases
        self.rotations = rotations
        self.simulation_generator = simulation_generator
        self.reciporical_radius = reciprocal_radius
        self.reciprocal_radius = reciprocal_radius
        self._spots = spots  # list of PhaseSpots, one per phase
        self._coords = [_PhaseCoordinates(p, s, r) for p, s, r in zip(plist, spots, rlist)]
        self.phase_index = 0
        self.rotation_index = 0

    # --- nesting as in the reference
    @property
    def coordinates(self):
        if self._multi_phase:
            return [c for c in self._coords]
        c = self._coords[0]
        if self.rotations.size == 1:
            return c[0]
        return c

    @property
    def has_multiple_phases(self):
        return self._multi_phase and len(self._coords) > 1

    @property
    def has_multiple_rotations(self):
        if self._multi_phase:
            return [r.size > 1 for r in self.rotations]
        return self.rotations.size > 1

    @property
    def num_phases(self):
        return len(self._coords) if self._multi_phase else 1

    @property
    def current_size(self):
        return len(self._coords[self.phase_index])

    @property
    def iphase(self):
        return _PhaseSelector(self)

    @property
    def irot(self):
        return _RotationSelector(self)

    @property
    def current_phase(self):
        return self.phases[self.phase_index] if self._multi_phase else self.phases

    def get_current_rotation_matrix(self):
        """3 x 3 matrix of the current rotation (``phase_index``, ``rotation_index``)."""
        rot = self.rotations[self.phase_index] if self._multi_phase else self.rotations
        return np.array(rot.to_matrix()[self.rotation_index])

    def deepcopy(self):
        """A copy with its own spot arrays (the generator is shared)."""
        return copy.deepcopy(self, {id(self.simulation_generator): self.simulation_generator})

    def rotate_shift_coordinates(self, angle: float, center=(0, 0), mirrored: bool = False):
        """The current pattern's spots turned in-plane by ``angle`` degrees
        (after a mirror across x when ``mirrored``) and shifted by
        ``center``: x + iy -> (x -/+ iy) e^{i angle} + c; z, intensities and
        hkl unchanged (diffsims/simulations/simulation2d.py:261-311)."""
        v = self.get_current_coordinates()
        data = v.data.copy()
        w = data[:, 0] + 1j * (-data[:, 1] if mirrored else data[:, 1])
        w = w * np.exp(1j * np.deg2rad(angle)) + complex(center[0], center[1])
        data[:, 0], data[:, 1] = w.real, w.imag
        return DiffractingVector(v.phase, data, v.intensity, v.hkl, v.rotation)

    def get_simulation(self, item):
        """(rotation, phase index, DiffractingVector) of flat index ``item``."""
        counts = np.cumsum([len(c) for c in self._coords])
        ind = int(np.searchsorted(counts, item, side="right"))
        start = 0 if ind == 0 else counts[ind - 1]
        c = self._coords[ind]
        return c.rotation[item - start], ind, c[item - start]

    def get_current_coordinates(self):
        return self._coords[self.phase_index][self.rotation_index]

    def __iter__(self):
        """The patterns in order, phase by phase, through the phase / rotation
        cursor as the reference iterates (the cursor is back at (0, 0) at
        the end)."""
        return self

    def __next__(self):
        if self.phase_index >= len(self._coords):
            self.phase_index = 0
            self.rotation_index = 0
            raise StopIteration
        v = self._coords[self.phase_index][self.rotation_index]
        if self.rotation_index + 1 >= self.current_size:
            self.rotation_index = 0
            self.phase_index += 1
        else:
            self.rotation_index += 1
        return v

    def __len__(self):
        return sum(len(c) for c in self._coords)

    def spots(self, phase_index=0):
        """Device CSR arrays of one phase (``PhaseSpots``)."""
        return self._spots[phase_index]

    def polar_flatten_simulations(self, radial_axes=None, azimuthal_axes=None, as_tensor=False, precision="fp64"):
        """(r, theta, intensity) templates padded to the largest pattern
        (diffsims/simulations/simulation2d.py:313-355), computed on the GPU
        (``ds_polar_flatten``).  numpy arrays as the reference returns them
        (int indices when both axes are given); ``as_tensor`` keeps float64
        device tensors instead.  ``precision='fp32'`` computes r and theta
        in FP32 (``ds_polar_flatten_f32``: ~2e-7 relative, many times
        faster on this GPU, whose FP64 rate is 1/64 of its FP32 rate)."""
        from .engine import polar_flatten
        r_t, t_t, i_t = polar_flatten(self._spots, radial_axes, azimuthal_axes, precision)
        if as_tensor:
            return r_t, t_t, i_t
        r_t, t_t, i_t = r_t.cpu().numpy(), t_t.cpu().numpy(), i_t.cpu().numpy()
        if radial_axes is not None and azimuthal_axes is not None:
            r_t = np.array(r_t, dtype=int)
            t_t = np.array(t_t, dtype=int)
        return r_t, t_t, i_t

    def get_diffraction_pattern(self, shape=None, sigma: float = 10, direct_beam_position=None,
                                in_plane_angle: float = 0, calibration: float = 0.01, mirrored: bool = False,
                                fast: bool = True, normalize: bool = True, clip_threshold: float = 1):
        """Detector image (rows, columns) of the current pattern
        (``phase_index``, ``rotation_index``), computed on the GPU
        (diffsims/simulations/simulation2d.py:357-442).  Returns a float64
        numpy array holding the kernel's float32 values."""
        from .engine import RasterSettings, rasterize
        settings = RasterSettings(shape, sigma, direct_beam_position, in_plane_angle, calibration, mirrored, fast,
                                  normalize, clip_threshold)
        spots = self._spots[self.phase_index]
        i = self.rotation_index if spots.n_orient > 1 else 0
        img = rasterize(spots, settings, i, i + 1)
        return img[0].cpu().numpy().astype(np.float64)

    def get_diffraction_patterns(self, shape, sigma: float = 10, direct_beam_position=None, in_plane_angle: float = 0,
                                 calibration: float = 0.01, mirrored: bool = False, fast: bool = True,
                                 normalize: bool = True, clip_threshold: float = 1, phase_index: int = 0,
                                 start: int = 0, stop=None, out=None, pixel_snap: float = 0.0):
        """Detector images of patterns ``start:stop`` of one phase in one
        launch: a float32 (n, rows, columns) tensor on the device (no
        counterpart in the reference, which loops over
        ``get_diffraction_pattern``).  ``out`` may be a preallocated tensor to
        stream chunks through."""
        from .engine import RasterSettings, rasterize
        settings = RasterSettings(shape, sigma, direct_beam_position, in_plane_angle, calibration, mirrored, fast,
                                  normalize, clip_threshold, pixel_snap=pixel_snap)
        return rasterize(self._spots[phase_index], settings, start, stop, out=out)

    def __repr__(self):
        return f"Simulation2D({self.num_phases} phase(s), {len(self)} pattern(s))"


def _get_closest(array, values):
    """Index of the closest entry of the sorted ``array`` for each value, the
    upper one on ties (diffsims/simulations/simulation2d.py:767-781)."""
    array = np.asarray(array)
    idxs = np.searchsorted(array, values, side="left")
    prev_closer = (idxs == len(array)) | (
        np.fabs(values - array[np.maximum(idxs - 1, 0)]) < np.fabs(values - array[np.minimum(idxs, len(array) - 1)]))
    idxs[prev_closer] -= 1
    return idxs


get_closest = _get_closest  # the reference's public name (simulation2d.py:767)
