"""FP64 CPU oracle for the per-family structure factors -- TEST INFRASTRUCTURE.

Restates, in numpy float64, diffsims/structure_factor/ (the EMsoft-derived
helpers): the Doyle-Turner parameter lookup
(atomic_scattering_parameters.py:145-244), the kinematical and Doyle-Turner
atomic scattering factors (atomic_scattering_factor.py:27-124), the family
structure factors (structure_factor.py:32-185) and the refraction-corrected
wavelength (structure_factor.py:188-233).  Only tests, ``smoke()`` and
``bench.py`` may import it; the ``diffsims_gb300`` package never does.

Third-party arithmetic restated here: diffpy.structure 3.0.2
(``expandPosition``, ``SymmetryConstraints``, ``Atom.Bisoequiv``,
``Lattice.volume``), called at structure_factor.py:30,88,94,155,162.
* ``expandPosition(sg, xyz)[0]``: the distinct positions ``R xyz + t``
  reduced into [0, 1) over the space group's operations (equal within 1e-5,
  modulo lattice translations).
* ``SymmetryConstraints(sg, positions).corepos``: the symmetry-independent
  positions in input order, so its first entry is ``positions[0]``;
  find_asymmetric_positions keeps only the mask of that first entry
  (the trailing ``[0]`` at structure_factor.py:49-52), so a structure factor
  sums the orbit of every atom equal to the first atom's position.
* ``Bisoequiv = 8 pi^2 Uisoequiv``; ``volume`` from the cell parameters.

Pinned by the reference's EMsoft-checked known answers
(diffsims/tests/structure_factor/test_structure_factor.py:79-181,
test_atomic_scattering_factor.py:27-110, test_atomic_scattering_parameters.py:25-70)
and by fixtures from running the reference's own structure_factor.py
(tests/golden/make_golden.py).
"""
from __future__ import annotations

import itertools
import json
import math
import pathlib
import re

import numpy as np
from scipy.constants import c as _C, e as _E, h as _H, physical_constants

_TABLES = json.loads(
    (pathlib.Path(__file__).resolve().parents[1] / "diffsims_gb300" / "data"
     / "scattering_params.json").read_text())
_DT = np.asarray(_TABLES["doyleturner"], dtype=np.float64)
_ELEMENTS = _TABLES["elements"]
_REST_MASS = physical_constants["atomic unit of mass"][0]


# ------------------------------------------------- parameters and elements
def element_id(symbol) -> int:
    """atomic_scattering_parameters.py:216-238 (the symbol -> Z map is built
    from ``zip(ELEMENTS, arange(1, 118))``, so Z = 118 has no entry)."""
    if not isinstance(symbol, str):
        return int(symbol)
    head = re.match("^(?P<element>[A-Za-z]*)", symbol).group("element").lower()
    table = dict(zip(_ELEMENTS, range(1, len(_ELEMENTS))))
    return table[head]


def element_symbol_from_id(z: int) -> str:
    """atomic_scattering_parameters.py:241-256."""
    table = dict(zip(range(1, len(_ELEMENTS)), _ELEMENTS))
    return table[z].capitalize()


def doyleturner_parameters(element, unit=None):
    """atomic_scattering_parameters.py:167-213: (a1-a4, b1-b4), x 1e-2 for nm."""
    z = element_id(element)
    factor = 1e-2 if (unit is not None and unit.lower() == "nm") else 1
    return _DT[z - 1, :4] * factor, _DT[z - 1, 4:] * factor


def atomic_f_kinematical(element, s, biso=0.0, occupancy=1.0):
    """atomic_scattering_factor.py:27-66."""
    z = element_id(element)
    a, b = doyleturner_parameters(z)
    s2 = s ** 2
    f = z - (41.78214 * s2 * np.sum(a * np.exp(-b * s2)))
    return f * (occupancy * np.exp(-biso * s2))


def atomic_f_doyleturner(element, s, volume, biso=0.0, occupancy=1.0):
    """atomic_scattering_factor.py:69-124."""
    a, b = doyleturner_parameters(element)
    s2 = s ** 2
    f = (47.87801 / volume) * np.sum(a * np.exp(-b * s2))
    return f * (occupancy * np.exp(-biso * s2))


def cell_volume(a, b, c, alpha, beta, gamma):
    ca, cb, cg = np.cos(np.deg2rad([alpha, beta, gamma]))
    return a * b * c * math.sqrt(1 + 2 * ca * cb * cg - ca * ca - cb * cb - cg * cg)


# ----------------------------------------------------------- space groups
def close_group(generators):
    """All (R, t mod 1) products of the generating operations."""
    def key(op):
        R, t = op
        return (tuple(np.rint(R).astype(int).ravel()), tuple(np.round(np.mod(t, 1.0) * 24).astype(int) % 24))

    ident = (np.eye(3), np.zeros(3))
    ops = {key(ident): ident}
    frontier = [ident]
    while frontier:
        new = []
        for (R1, t1), (R2, t2) in itertools.product(frontier, generators):
            op = (R2 @ R1, np.mod(R2 @ t1 + t2, 1.0))
            k = key(op)
            if k not in ops:
                ops[k] = op
                new.append(op)
        frontier = new
    return list(ops.values())


def _m(rows):
    return np.array(rows, dtype=np.float64)


_C4Z = _m([[0, -1, 0], [1, 0, 0], [0, 0, 1]])
_C3D = _m([[0, 0, 1], [1, 0, 0], [0, 1, 0]])
_INV = -np.eye(3)
_C3Z_HEX = _m([[0, -1, 0], [1, -1, 0], [0, 0, 1]])
_C2Z = _m([[-1, 0, 0], [0, -1, 0], [0, 0, 1]])
_MXY_HEX = _m([[0, -1, 0], [-1, 0, 0], [0, 0, 1]])


def space_group_operations(number: int):
    """Operations (R, t) of the space groups the tests use, generated here
    from their standard generators (International Tables A, origin choice of
    the reference's test phases): 1 P1, 2 P-1, 186 P6_3mc, 221 Pm-3m,
    225 Fm-3m, 229 Im-3m."""
    z = np.zeros(3)
    if number == 1:
        return close_group([])
    if number == 2:
        return close_group([(_INV, z)])
    if number == 186:
        return close_group([(_C3Z_HEX, z), (_C2Z, np.array([0, 0, 0.5])), (_MXY_HEX, z)])
    cubic = [(_C4Z, z), (_C3D, z), (_INV, z)]
    if number == 221:
        return close_group(cubic)
    if number == 225:
        return close_group(cubic + [(np.eye(3), np.array(t)) for t in ([0, .5, .5], [.5, 0, .5])])
    if number == 229:
        return close_group(cubic + [(np.eye(3), np.array([.5, .5, .5]))])
    raise KeyError(f"space group {number} is not tabulated in the oracle")


def orbit(ops, xyz, eps=1e-5):
    """expandPosition(sg, xyz)[0]: distinct images R xyz + t in [0, 1)."""
    out = []
    xyz = np.asarray(xyz, dtype=np.float64)
    for R, t in ops:
        p = R @ xyz + t
        p = p - np.floor(p)
        if any(np.all(np.abs((p - q) - np.rint(p - q)) < eps) for q in out):
            continue
        out.append(p)
    return np.array(out)


def asymmetric_mask(positions):
    """find_asymmetric_positions (structure_factor.py:32-52) with corepos[0] =
    positions[0]: the atoms equal (np.allclose) to the first position."""
    positions = [np.asarray(p, dtype=np.float64) for p in positions]
    return np.array([np.allclose(p, positions[0]) for p in positions])


# -------------------------------------------------- family structure factors
def family_structure_factor(atoms, ops, hkl, s, kind, volume=None):
    """Complex F of one family (structure_factor.py:55-100 for kind
    "kinematical", :103-166 before the relativistic epilogue for
    "doyleturner"), in the reference's order: asymmetric atoms, then their
    orbits, F += f exp(-2 pi i h.x).  ``atoms``: (element, xyz, occupancy,
    Bisoequiv) tuples."""
    hkl = np.asarray(hkl, dtype=np.float64)
    mask = asymmetric_mask([a[1] for a in atoms])
    F = 0 + 0j
    for keep, (el, xyz, occ, biso) in zip(mask, atoms):
        if not keep:
            continue
        if kind == "kinematical":
            f = atomic_f_kinematical(el, s, biso, occ)
        else:
            f = atomic_f_doyleturner(el, s, volume, biso, occ)
        for p in orbit(ops, xyz):
            arg = 2 * np.pi * np.sum(hkl * p)
            F += f * (np.cos(arg) - np.sin(arg) * 1j)
    return F


def kinematical_structure_factor(atoms, ops, hkl, s):
    """get_kinematical_structure_factor (structure_factor.py:55-100): Re F."""
    return family_structure_factor(atoms, ops, hkl, s, "kinematical").real


def doyleturner_structure_factor(atoms, ops, hkl, s, volume, voltage):
    """get_doyleturner_structure_factor (structure_factor.py:103-185):
    returns (value, params)."""
    F = family_structure_factor(atoms, ops, hkl, s, "doyleturner", volume)
    gamma = 1 + (2 * _E * 0.5 * voltage / _REST_MASS / (_C ** 2))
    v_mod = abs(F) * gamma
    v_phase = np.arctan2(F.imag, F.real)
    v_g = v_mod * np.exp(v_phase * 1j)
    pre = 2 * (_REST_MASS * _E / _H ** 2) * 1e-18
    return (pre * v_g).real, {"gamma_relcor": gamma, "v_mod": v_mod, "v_phase": v_phase, "v_g": v_g}


def refraction_corrected_wavelength(atoms, ops, volume, voltage):
    """get_refraction_corrected_wavelength (structure_factor.py:188-233)."""
    temp1 = 1e9 * _H / np.sqrt(2 * _REST_MASS * _E)
    temp2 = _E * 0.5 * voltage / _REST_MASS / (_C ** 2)
    psi_hat = voltage * (1 + temp2)
    _, params = doyleturner_structure_factor(atoms, ops, np.zeros(3, dtype=int), 0, volume, voltage)
    psi_hat += params["v_mod"]
    return temp1 / np.sqrt(psi_hat)
