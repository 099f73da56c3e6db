"""diffsims' own result types over GPU results.

Callers of ``SimulationGenerator.calculate_diffraction2d`` such as pyxem's
template matching receive, from the reference, a
``diffsims.simulations.Simulation2D`` whose coordinates are
``diffsims.crystallography.DiffractingVector`` objects
(diffsims/generators/simulation_generator.py:244-258).  When that package
(with orix and diffpy) is importable, ``to_reference_simulation`` gives the
same types for a result of this library:

* the object is an instance of the reference's ``Simulation2D`` (a subclass
  created here), so type checks, iteration, slicing (``iphase``, ``irot``),
  ``get_simulation``, ``rotate_shift_coordinates`` and plotting run the
  reference's own code;
* its coordinates are built per pattern the first time that pattern is read,
  from the device CSR spots, the way the reference builds them
  (diffsims/generators/simulation_generator.py:319-385,
  diffsims/crystallography/_diffracting_vector.py:84-161): a deep copy of
  the phase whose lattice basis rotation is multiplied by the pattern's
  rotation matrix (``baserot @ R``), the beam-frame spot vectors as ``xyz``,
  and the intensities;
* ``polar_flatten_simulations`` and ``get_diffraction_pattern`` run the GPU
  kernels of this library (the reference's versions would build every
  vector first); their results are the native ``Simulation2D``'s.

Without the reference package the native ``Simulation2D`` (same nesting and
attributes, lazy per-pattern ``DiffractingVector`` views) is the result.
"""
from __future__ import annotations

import sys

import numpy as np

_SUBCLASSES = {}


def reference_classes():
    """(Simulation2D, DiffractingVector) of the reference package, or None
    when it (or orix / diffpy, which it imports) is not importable."""
    try:
        from diffsims.crystallography import DiffractingVector
        from diffsims.simulations import Simulation2D
    except Exception:  # ImportError, or an import-time error of a missing dependency
        return None
    return Simulation2D, DiffractingVector


_CLASSES = []


def cached_reference_classes():
    """``reference_classes()``, looked up once per process."""
    if not _CLASSES:
        _CLASSES.append(reference_classes())
    return _CLASSES[0]


def reference_vector(vector_cls, phase, rotation, xyz, intensity):
    """One pattern as the reference's DiffractingVector: the phase deep-copied
    with its lattice basis turned by ``rotation`` (a single rotation with
    ``to_matrix``), the spot vectors ``xyz`` (n, 3) and their intensities."""
    rotated = phase.deepcopy()
    lattice = rotated.structure.lattice
    R = np.asarray(rotation.to_matrix(), dtype=np.float64).reshape(3, 3)
    lattice.setLatPar(baserot=lattice.baserot @ R)
    v = vector_cls(rotated, xyz=np.asarray(xyz, dtype=np.float64).reshape(-1, 3))
    v.intensity = np.asarray(intensity, dtype=np.float64)
    return v


class LazyPatterns:
    """The patterns of one phase as reference DiffractingVectors, each built
    (and kept) the first time it is read.  Indexing with an integer gives one
    vector; with a slice, list or array, an object array of vectors (as
    indexing the reference's object array does); ``np.array(...)`` builds
    them all."""

    def __init__(self, spots, phase, rotation, vector_cls):
        self._spots = spots
        self._phase = phase
        self._rotation = rotation
        self._cls = vector_cls
        self._built = {}

    def __len__(self):
        return int(self._spots.n_orient)

    @property
    def size(self):
        return len(self)

    @property
    def shape(self):
        return (len(self),)

    def _one(self, i):
        v = self._built.get(i)
        if v is None:
            _, xyz, inten = self._spots.pattern(i)
            v = reference_vector(self._cls, self._phase, self._rotation[i], xyz, inten)
            self._built[i] = v
        return v

    def __getitem__(self, key):
        if isinstance(key, (int, np.integer)):
            n = len(self)
            i = int(key) + n if key < 0 else int(key)
            if not 0 <= i < n:
                raise IndexError(key)
            return self._one(i)
        idx = np.arange(len(self))[key]
        out = np.empty(idx.shape[0], dtype=object)
        for j, i in enumerate(idx):
            out[j] = self._one(int(i))
        return out

    def __iter__(self):
        for i in range(len(self)):
            yield self._one(i)

    def __array__(self, dtype=None, copy=None):
        return self[:]


def _subclass_of(sim_cls):
    """A subclass of the reference's Simulation2D that keeps lazy pattern
    sequences (its constructor would turn them into object arrays, building
    every vector) and runs the GPU kernels for templates and images."""
    cls = _SUBCLASSES.get(sim_cls)
    if cls is not None:
        return cls
    mod = sys.modules.get(sim_cls.__module__)

    def __init__(self, phases, coordinates, rotations, simulation_generator, reciprocal_radius=1.0, native=None):
        # what the reference's constructor sets (simulation2d.py:115-198)
        self.phases = phases
        self.rotations = rotations
        self.coordinates = coordinates
        self.simulation_generator = simulation_generator
        self.phase_index = 0
        self.rotation_index = 0
        self._rot_plot = None
        self._diff_plot = None
        self.reciporical_radius = reciprocal_radius
        if mod is not None and hasattr(mod, "PhaseGetter"):
            self.iphase = mod.PhaseGetter(self)
            self.irot = mod.RotationGetter(self)
        self._rotation_slider = None
        self._phase_slider = None
        self._native = native

    def polar_flatten_simulations(self, radial_axes=None, azimuthal_axes=None):
        """(r, theta, intensity) templates of every pattern, computed on the
        GPU (diffsims/simulations/simulation2d.py:313-355)."""
        return self._native.polar_flatten_simulations(radial_axes, azimuthal_axes)

    def get_diffraction_pattern(self, shape=None, sigma=10, direct_beam_position=None, in_plane_angle=0,
                                calibration=0.01, mirrored=False, fast=True, normalize=True, clip_threshold=1):
        """Detector image of the current pattern, rasterised on the GPU
        (diffsims/simulations/simulation2d.py:357-442)."""
        self._native.phase_index, self._native.rotation_index = self.phase_index, self.rotation_index
        return self._native.get_diffraction_pattern(shape, sigma, direct_beam_position, in_plane_angle, calibration,
                                                    mirrored, fast, normalize, clip_threshold)

    cls = type(sim_cls.__name__, (sim_cls,), {
        "__init__": __init__, "polar_flatten_simulations": polar_flatten_simulations,
        "get_diffraction_pattern": get_diffraction_pattern, "__module__": __name__,
        "__doc__": f"{sim_cls.__name__} of the reference over device spots (diffsims_gb300)."})
    _SUBCLASSES[sim_cls] = cls
    return cls


def to_reference_simulation(sim, phases, rotations, classes=None):
    """The reference's ``Simulation2D`` for a native result ``sim`` of
    ``calculate_diffraction2d``.  ``phases`` and ``rotations`` are the
    caller's own objects (orix ``Phase`` and ``Rotation``), nested as the
    caller passed them (one phase and its rotations, or sequences of both).
    ``classes``: (Simulation2D, DiffractingVector), by default the reference
    package's (``reference_classes``)."""
    classes = classes or reference_classes()
    if classes is None:
        raise ImportError("the diffsims package (with orix and diffpy) is not importable")
    sim_cls, vec_cls = classes
    multi = isinstance(phases, (list, tuple))
    plist = list(phases) if multi else [phases]
    rlist = list(rotations) if multi else [rotations]
    coords = []
    for k, (p, r) in enumerate(zip(plist, rlist)):
        lazy = LazyPatterns(sim.spots(k), p, r, vec_cls)
        coords.append(lazy[0] if getattr(r, "size", len(lazy)) == 1 and not multi else lazy)
    if multi:
        return _subclass_of(sim_cls)(plist, coords, rlist, sim.simulation_generator, sim.reciprocal_radius, sim)
    return _subclass_of(sim_cls)(plist[0], coords[0], rlist[0], sim.simulation_generator, sim.reciprocal_radius, sim)
