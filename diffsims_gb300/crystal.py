"""Minimal phase / structure / rotation types accepted by the drop-in API.

The reference takes orix ``Phase`` (with a diffpy ``Structure``) and orix
``Rotation`` objects (diffsims/generators/simulation_generator.py:134-146).
Neither library is needed here: these small classes carry the same
information, and the adapters below also accept the real orix / diffpy objects
by duck typing (``phase.structure.lattice`` with a, b, c, alpha, beta, gamma;
sites with ``element``, ``xyz``, ``occupancy``; ``rotation.data`` quaternions).

Lattice frame: x || a, z || c* (b in the xy-plane) -- the frame orix ``Phase``
imposes on every structure, in which the reference's beam-frame coordinates
are expressed.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np


@dataclass
class Lattice:
    a: float
    b: float
    c: float
    alpha: float = 90.0
    beta: float = 90.0
    gamma: float = 90.0

    def abcABG(self):
        return (self.a, self.b, self.c, self.alpha, self.beta, self.gamma)

    @property
    def base(self) -> np.ndarray:
        """Direct base vectors (rows a, b, c) in the x || a, z || c* frame."""
        return lattice_base(*self.abcABG())

    @property
    def stdbase(self):
        return self.base

    @property
    def recbase(self):
        return np.linalg.inv(self.base)

    @property
    def volume(self) -> float:
        """Cell volume (Angstrom^3), as diffpy ``Lattice.volume``."""
        ca, cb, cg = np.cos(np.deg2rad([self.alpha, self.beta, self.gamma]))
        return float(self.a * self.b * self.c * math.sqrt(1 + 2 * ca * cb * cg - ca * ca - cb * cb - cg * cg))

    @property
    def reciprocal_base(self) -> np.ndarray:
        """Rows a*, b*, c* (no 2 pi): g = hkl @ reciprocal_base."""
        return np.linalg.inv(self.base).T


def _check_cell(a, b, c, alpha, beta, gamma):
    p = np.array([a, b, c, alpha, beta, gamma], dtype=np.float64)
    if not (np.all(np.isfinite(p)) and np.all(p[:3] > 0) and np.all((p[3:] > 0) & (p[3:] < 180))):
        raise ValueError(f"invalid lattice: a={a} b={b} c={c} alpha={alpha} beta={beta} gamma={gamma}")


def lattice_base(a, b, c, alpha, beta, gamma) -> np.ndarray:
    _check_cell(a, b, c, alpha, beta, gamma)
    al, be, ga = np.deg2rad([alpha, beta, gamma])
    ca, cb, cg, sg = np.cos(al), np.cos(be), np.cos(ga), np.sin(ga)
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz2 = c * c - cx * cx - cy * cy
    if not cz2 > 0:
        raise ValueError(f"degenerate lattice: a={a} b={b} c={c} alpha={alpha} beta={beta} gamma={gamma}")
    return np.array([[a, 0.0, 0.0], [b * cg, b * sg, 0.0], [cx, cy, math.sqrt(cz2)]])


def diffpy_base(a, b, c, alpha, beta, gamma) -> np.ndarray:
    """Direct base vectors (rows a, b, c) in diffpy's standard Cartesian frame,
    the frame of diffpy ``Structure`` objects and of the legacy
    ``DiffractionGenerator``: c along z, b in the yz-plane (so a* is along x).
    Built from the cell geometry: b = b (0, sin alpha, cos alpha); a_z from
    a.c, a_y from a.b, a_x > 0 from |a|."""
    _check_cell(a, b, c, alpha, beta, gamma)
    al, be, ga = np.deg2rad([alpha, beta, gamma])
    bv = np.array([0.0, b * math.sin(al), b * math.cos(al)])
    az = a * math.cos(be)
    ay = (a * b * math.cos(ga) - az * bv[2]) / bv[1]
    ax2 = a * a - ay * ay - az * az
    if not ax2 > 0:
        raise ValueError(f"degenerate lattice: a={a} b={b} c={c} alpha={alpha} beta={beta} gamma={gamma}")
    return np.array([[math.sqrt(ax2), ay, az], bv, [0.0, 0.0, c]])


@dataclass
class Atom:
    element: str
    xyz: Sequence[float]
    occupancy: float = 1.0
    Uisoequiv: float = 0.0

    def __post_init__(self):
        self.xyz = np.asarray(self.xyz, dtype=np.float64)

    @property
    def Bisoequiv(self) -> float:
        """Isotropic Debye-Waller B = 8 pi^2 U (Angstrom^2), as diffpy ``Atom``."""
        return 8 * math.pi ** 2 * self.Uisoequiv


class Structure(list):
    """A list of ``Atom`` with a ``lattice`` (the diffpy Structure surface the
    reference reads: iteration over sites and ``structure.lattice``)."""

    def __init__(self, atoms=(), lattice: Lattice | None = None):
        super().__init__(atoms)
        self.lattice = lattice if lattice is not None else Lattice(1, 1, 1)


@dataclass
class Phase:
    name: str = ""
    structure: Structure = field(default_factory=Structure)
    space_group: int | None = None
    point_group: str | None = None


# ----------------------------------------------------------------- rotations
def euler_to_quaternion(euler, degrees: bool = False) -> np.ndarray:
    """Bunge (phi1, Phi, phi2) -> unit quaternions (w, x, y, z), w >= 0.

    Passive convention with P = +1 of Rowenhorst et al., Modelling Simul.
    Mater. Sci. Eng. 23 (2015) 083501, as orix ``Rotation.from_euler``.
    """
    e = np.atleast_2d(np.asarray(euler, dtype=np.float64))
    if degrees:
        e = np.deg2rad(e)
    s1, s2 = 0.5 * (e[:, 0] + e[:, 2]), 0.5 * (e[:, 0] - e[:, 2])
    c, s = np.cos(e[:, 1] / 2), np.sin(e[:, 1] / 2)
    q = np.stack([c * np.cos(s1), -s * np.cos(s2), -s * np.sin(s2), -c * np.sin(s1)], axis=1)
    q[q[:, 0] < 0] *= -1
    return q


class Rotation:
    """Unit quaternions (w, x, y, z), shape (N, 4): the active rotation of the
    crystal, as orix ``Rotation``."""

    def __init__(self, data):
        q = np.asarray(data, dtype=np.float64).reshape(-1, 4)
        n = np.linalg.norm(q, axis=1, keepdims=True)
        if np.any(n == 0) or not np.all(np.isfinite(q)):
            raise ValueError("rotations must be finite, non-zero quaternions")
        self.data = q / n

    @classmethod
    def from_euler(cls, euler, degrees: bool = False):
        return cls(euler_to_quaternion(euler, degrees))

    @classmethod
    def identity(cls, n: int = 1):
        q = np.zeros((n, 4))
        q[:, 0] = 1
        return cls(q)

    @classmethod
    def random(cls, n: int = 1, seed=None):
        """Uniform on SO(3): normalised standard-normal 4-vectors, w >= 0."""
        rng = np.random.default_rng(seed)
        q = rng.standard_normal((n, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        q[q[:, 0] < 0] *= -1
        return cls(q)

    @property
    def size(self) -> int:
        return self.data.shape[0]

    @property
    def shape(self):
        return (self.size,)

    def __len__(self):
        return self.size

    def __getitem__(self, key):
        return Rotation(self.data[key])

    def to_matrix(self) -> np.ndarray:
        w, x, y, z = self.data.T
        return np.stack([
            np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
            np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
            np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
        ], axis=1)

    def __repr__(self):
        return f"Rotation {self.shape}"


# ------------------------------------------------------------------ adapters
def lattice_params(lattice) -> tuple:
    if hasattr(lattice, "abcABG"):
        return tuple(float(v) for v in lattice.abcABG())
    return tuple(float(getattr(lattice, k)) for k in ("a", "b", "c", "alpha", "beta", "gamma"))


def structure_of(phase):
    return phase.structure if hasattr(phase, "structure") else phase


def sites_of(structure):
    """(elements, xyz (N,3), occupancy (N,)) of a structure-like object."""
    els, xyz, occ = [], [], []
    for site in structure:
        els.append(str(site.element))
        xyz.append(site.xyz)
        occ.append(getattr(site, "occupancy", 1.0))
    if not els:
        raise ValueError("the structure has no atoms")
    return els, np.asarray(xyz, dtype=np.float64).reshape(-1, 3), np.asarray(occ, dtype=np.float64)


def quaternions_of(rotation) -> np.ndarray:
    """(N, 4) float64 quaternions from a Rotation / orix Rotation / array."""
    if hasattr(rotation, "data"):
        q = np.asarray(rotation.data, dtype=np.float64)
    else:
        q = np.asarray(rotation, dtype=np.float64)
    q = q.reshape(-1, 4)
    return np.ascontiguousarray(q)
