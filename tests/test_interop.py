"""The reference result types over GPU results (``diffsims_gb300.interop``),
on CPU with duck-typed stand-ins: orix ``Phase`` (deep copy, a diffpy
lattice with ``baserot`` / ``setLatPar``), orix ``Rotation`` (``size``,
indexing, ``to_matrix``), diffsims' ``DiffractingVector`` and a base
``Simulation2D`` class whose methods read ``coordinates`` the way the
reference's do.  The native result is replaced by a stand-in holding host
patterns, so no GPU is needed.
"""
import copy

import numpy as np
import pytest

from diffsims_gb300 import interop


class FakeLattice:
    def __init__(self):
        self.baserot = np.eye(3)

    def setLatPar(self, baserot=None):
        self.baserot = np.array(baserot)


class FakeStructure:
    def __init__(self):
        self.lattice = FakeLattice()


class FakePhase:
    def __init__(self, name):
        self.name = name
        self.structure = FakeStructure()
        self.copies = 0

    def deepcopy(self):
        self.copies += 1
        return copy.deepcopy(self)


def _rot(angle):
    c, s = np.cos(angle), np.sin(angle)
    return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])


class FakeRotation:
    def __init__(self, angles):
        self.angles = np.atleast_1d(np.asarray(angles, dtype=np.float64))

    @property
    def size(self):
        return self.angles.size

    def __getitem__(self, i):
        return FakeRotation(self.angles[i])

    def to_matrix(self):
        return np.stack([_rot(a) for a in self.angles])


class FakeVector:
    """DiffractingVector stand-in: (phase, xyz) and an intensity setter."""

    def __init__(self, phase, xyz=None):
        self.phase = phase
        self.data = np.asarray(xyz)
        self._intensity = np.full(self.data.shape[0], np.nan)

    @property
    def size(self):
        return self.data.shape[0]

    @property
    def intensity(self):
        return self._intensity

    @intensity.setter
    def intensity(self, v):
        self._intensity = np.asarray(v)


class FakeReferenceSimulation:
    """Base class standing in for diffsims' Simulation2D: its constructor
    would build object arrays, which the subclass must not call; its
    ``get_simulation`` reads ``coordinates`` as the reference does."""

    def __init__(self, *a, **k):
        raise AssertionError("the reference constructor must not run (it would build every vector)")

    def get_simulation(self, item):
        if isinstance(self.phases, list):
            counts = np.cumsum([r.size for r in self.rotations])
            ind = int(np.searchsorted(counts, item, side="right"))
            start = 0 if ind == 0 else counts[ind - 1]
            return self.rotations[ind][item - start], ind, self.coordinates[ind][item - start]
        return self.rotations[item], 0, self.coordinates[item]


class FakeSpots:
    def __init__(self, patterns):
        self._p = patterns
        self.read = []

    @property
    def n_orient(self):
        return len(self._p)

    def pattern(self, i):
        self.read.append(i)
        xyz, inten = self._p[i]
        return np.zeros((len(inten), 3), np.int32), xyz, inten


class FakeNative:
    def __init__(self, spots_list):
        self._spots = spots_list
        self.simulation_generator = "gen"
        self.reciprocal_radius = 1.5
        self.phase_index = self.rotation_index = 0

    def spots(self, k=0):
        return self._spots[k]

    def polar_flatten_simulations(self, radial_axes=None, azimuthal_axes=None):
        return "templates", radial_axes, azimuthal_axes


def _patterns(n, seed):
    rng = np.random.default_rng(seed)
    return [(rng.normal(size=(k, 3)), rng.random(k)) for k in rng.integers(0, 6, n)]


CLASSES = (FakeReferenceSimulation, FakeVector)


def test_single_phase_many_rotations_builds_vectors_lazily():
    pats = _patterns(7, 1)
    spots = FakeSpots(pats)
    phase = FakePhase("p")
    rot = FakeRotation(np.linspace(0, 1, 7))
    sim = interop.to_reference_simulation(FakeNative([spots]), phase, rot, classes=CLASSES)
    assert isinstance(sim, FakeReferenceSimulation)
    assert spots.read == [] and phase.copies == 0          # nothing built yet
    assert sim.reciporical_radius == 1.5 and sim.simulation_generator == "gen"
    r, ind, v = sim.get_simulation(3)
    assert spots.read == [3] and ind == 0
    assert isinstance(v, FakeVector)
    np.testing.assert_array_equal(v.data, pats[3][0])
    np.testing.assert_array_equal(v.intensity, pats[3][1])
    # the vector's phase is a rotated deep copy: baserot = I @ R(angle_3)
    np.testing.assert_allclose(v.phase.structure.lattice.baserot, _rot(rot.angles[3]))
    np.testing.assert_array_equal(phase.structure.lattice.baserot, np.eye(3))  # the caller's phase is untouched
    assert sim.coordinates[3] is v                                           # built once, kept
    arr = sim.coordinates[1:4]
    assert arr.dtype == object and arr.shape == (3,) and arr[2] is v
    assert len(np.array(sim.coordinates, dtype=object)) == 7
    assert sim.polar_flatten_simulations([1, 2], [3]) == ("templates", [1, 2], [3])


def test_single_phase_single_rotation_is_one_vector():
    pats = _patterns(1, 2)
    sim = interop.to_reference_simulation(FakeNative([FakeSpots(pats)]), FakePhase("p"), FakeRotation([0.3]),
                                          classes=CLASSES)
    assert isinstance(sim.coordinates, FakeVector)
    np.testing.assert_array_equal(sim.coordinates.data, pats[0][0])


def test_multi_phase_nesting():
    a, b = _patterns(2, 3), _patterns(1, 4)
    phases = [FakePhase("a"), FakePhase("b")]
    rots = [FakeRotation([0.1, 0.2]), FakeRotation([0.5])]
    sim = interop.to_reference_simulation(FakeNative([FakeSpots(a), FakeSpots(b)]), phases, rots, classes=CLASSES)
    assert isinstance(sim.coordinates, list) and len(sim.coordinates) == 2
    assert len(sim.coordinates[1]) == 1          # a list per phase even for one rotation, as the reference
    r, ind, v = sim.get_simulation(2)
    assert ind == 1
    np.testing.assert_array_equal(v.data, b[0][0])
    np.testing.assert_allclose(v.phase.structure.lattice.baserot, _rot(0.5))


def test_missing_reference_package_raises():
    if interop.reference_classes() is not None:
        pytest.skip("the reference package is importable here")
    with pytest.raises(ImportError):
        interop.to_reference_simulation(FakeNative([FakeSpots([])]), FakePhase("p"), FakeRotation([0.0]))
