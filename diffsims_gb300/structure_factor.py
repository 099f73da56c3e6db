"""Structure factors of lattice-plane families on the GPU.

Mirrors the public functions of diffsims/structure_factor/ (the helpers the
reference adapted from EMsoft): ``get_kinematical_structure_factor``,
``get_doyleturner_structure_factor``, ``get_refraction_corrected_wavelength``,
``find_asymmetric_positions``, the two atomic scattering factors and the
Doyle-Turner parameter lookup -- same names, argument meaning, return values
and errors.  The reference evaluates one family per call in a Python loop
over atoms; here ``hkl`` may also be an ``(N, 3)`` array and
``scattering_parameter`` an ``(N,)`` array, and all N families go to the GPU
in one launch (``ds_family_structure_factors``, FP64).  Scalar inputs give
scalar results, as in the reference.

Space groups: the orbit of each position is ``{R xyz + t}`` reduced into
[0, 1) over the space group's operations, distinct within 1e-5 (diffpy's
``expandPosition``).  ``phase.space_group`` may be a diffpy ``SpaceGroup``
(what an orix ``Phase`` carries), any object with ``iter_symops()`` or
``symop_list`` of operations with ``R`` and ``t``, a sequence of ``(R, t)``
pairs, or ``None`` / ``1`` (P1).  Other space-group numbers need their
operations from one of those forms.
"""
from __future__ import annotations

import math
import re

import numpy as np
import torch
from scipy.constants import c as _C, e as _E, h as _H, physical_constants

from . import _native as N
from .sim_utils import PackedAtoms, _TABLES
from .crystal import sites_of
from .engine import reciprocal_basis
from .symmetry import expand_position, point_group_rotations, symmetry_families

__all__ = [
    "get_doyleturner_atomic_scattering_factor",
    "get_kinematical_atomic_scattering_factor",
    "get_atomic_scattering_parameters",
    "get_element_id_from_string",
    "find_asymmetric_positions",
    "get_doyleturner_structure_factor",
    "get_kinematical_structure_factor",
    "get_refraction_corrected_wavelength",
    "calculate_structure_factor",
]

ELEMENTS = list(_TABLES["elements"])
N_ELEMENTS = len(ELEMENTS)
ATOMIC_SCATTERING_PARAMETERS_DOYLETURNER = np.asarray(_TABLES["doyleturner"], dtype=np.float64)
_REST_MASS = physical_constants["atomic unit of mass"][0]


# ------------------------------------------------------------- elements
def get_element(atom_type_symbol):
    """Alphabetic head of a CIF atom type symbol
    (diffsims/structure_factor/atomic_scattering_parameters.py:145-164)."""
    return re.match("^(?P<element>[A-Za-z]*)", atom_type_symbol).group("element")


def get_element_id_from_string(element_str):
    """Atomic number of an element symbol (atomic_scattering_parameters.py:216-238).
    Unknown symbols raise ``KeyError``; the map pairs ``ELEMENTS`` with 1..117,
    as the reference's ``zip`` does."""
    element2periodic = dict(zip(ELEMENTS[:N_ELEMENTS], range(1, N_ELEMENTS)))
    return element2periodic[get_element(element_str).lower()]


def _get_string_from_element_id(element_id):
    """Capitalised symbol of an atomic number (atomic_scattering_parameters.py:241-256)."""
    periodic2element = dict(zip(range(1, N_ELEMENTS), ELEMENTS[:N_ELEMENTS]))
    return periodic2element[element_id].capitalize()


def _element_id(element):
    return get_element_id_from_string(element) if isinstance(element, str) else int(element)


def get_atomic_scattering_parameters(element, unit=None):
    """Doyle-Turner a1-a4, b1-b4 for Z = 1-98 in 1/Angstrom^2, or 1/nm^2 x 1e-2
    with ``unit="nm"`` (atomic_scattering_parameters.py:167-213)."""
    factor = 1e-2 if (unit is not None and unit.lower() == "nm") else 1
    row = ATOMIC_SCATTERING_PARAMETERS_DOYLETURNER[_element_id(element) - 1]
    return row[:4] * factor, row[4:] * factor


def find_asymmetric_positions(positions, space_group):
    """Mask of the positions equal to the first symmetry-independent one
    (diffsims/structure_factor/structure_factor.py:32-52).  The reference takes
    the first entry of diffpy's ``SymmetryConstraints(...).corepos``, which is
    the first position, and keeps only that entry's mask; the structure
    factors below therefore sum the orbits of the atoms at the first atom's
    position, as the reference's do."""
    positions = [np.asarray(p, dtype=np.float64) for p in positions]
    if not positions:
        raise IndexError("find_asymmetric_positions: no positions")
    return np.array([np.allclose(p, positions[0]) for p in positions])


# ----------------------------------------------------------- GPU core
def _biso(atom):
    if hasattr(atom, "Bisoequiv"):
        return float(atom.Bisoequiv)
    return 8 * math.pi ** 2 * float(getattr(atom, "Uisoequiv", 0.0))


def _volume(lattice):
    if hasattr(lattice, "volume"):
        v = lattice.volume
        return float(v() if callable(v) else v)
    a, b, c, al, be, ga = (float(getattr(lattice, k)) for k in ("a", "b", "c", "alpha", "beta", "gamma"))
    ca, cb, cg = np.cos(np.deg2rad([al, be, ga]))
    return a * b * c * math.sqrt(1 + 2 * ca * cb * cg - ca * ca - cb * cb - cg * cg)


def _coeff_row(element_id, kind, volume):
    a, b = get_atomic_scattering_parameters(element_id)
    row = np.zeros(10)
    row[0:8:2], row[1:8:2] = a, b
    row[8] = float(element_id) if kind == N.DS_SCATTER_KINEMATICAL else 47.87801 / volume
    return row


def _family_F(sites, hkl, s, kind, volume):
    """Complex F (reference sign, exp(-2 pi i h.x)) of N families on the device.
    ``sites``: (element id, [orbit positions], occupancy, Bisoequiv)."""
    lib = N.load_library()
    dev = torch.device("cuda", torch.cuda.current_device())
    species, rows, index, xyz, occ, B = [], [], {}, [], [], []
    for z, positions, o, biso in sites:
        if z not in index:
            index[z] = len(rows)
            rows.append(_coeff_row(z, kind, volume))
        for p in positions:
            species.append(index[z])
            xyz.append(p)
            occ.append(o)
            B.append(4.0 * biso)  # the kernel's Debye-Waller term is exp(-B s^2 / 4)
    atoms = PackedAtoms.from_rows(species, rows, np.asarray(xyz), occ, B, kind, dev)
    n = hkl.shape[0]
    hkl_t = torch.as_tensor(np.ascontiguousarray(hkl, dtype=np.float64)).to(dev)
    s_t = torch.as_tensor(np.ascontiguousarray(s, dtype=np.float64)).to(dev)
    F = torch.empty((n, 2), dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    N.check(lib.ds_family_structure_factors(atoms.cstruct(), N.ptr(hkl_t), N.ptr(s_t), n, N.ptr(F), N.ptr(status),
                                            N.stream_handle()), "family structure factors")
    N.check_device_status(status, "family structure factors")
    return torch.complex(F[:, 0], -F[:, 1])


def _families(hkl, scattering_parameter):
    """(hkl (N, 3), s (N,), scalar?) from one family or arrays of families."""
    h = np.asarray(hkl, dtype=np.float64)
    scalar = h.ndim == 1
    h = h.reshape(-1, 3)
    s = np.broadcast_to(np.asarray(scattering_parameter, dtype=np.float64).reshape(-1), (h.shape[0],)).copy()
    return h, s, scalar


def _asymmetric_sites(structure, space_group):
    atoms = list(structure)
    mask = find_asymmetric_positions([a.xyz for a in atoms], space_group)
    return [(_element_id(a.element), expand_position(space_group, a.xyz), float(getattr(a, "occupancy", 1.0)),
             _biso(a)) for keep, a in zip(mask, atoms) if keep]


def _out(x: torch.Tensor, scalar: bool):
    v = x.cpu().numpy()
    return v[0] if scalar else v


# --------------------------------------------------------- public API
def get_kinematical_structure_factor(phase, hkl, scattering_parameter):
    """Kinematical (X-ray) structure factor Re F of the family hkl
    (diffsims/structure_factor/structure_factor.py:55-100): the orbit sum of
    ``f = Z - 41.78214 s^2 sum_i a_i exp(-b_i s^2)`` times occupancy and
    ``exp(-Bisoequiv s^2)``.  ``hkl`` (3,) or (N, 3), ``scattering_parameter``
    s = 1/(2d), scalar or (N,)."""
    h, s, scalar = _families(hkl, scattering_parameter)
    sites = _asymmetric_sites(phase.structure, phase.space_group)
    F = _family_F(sites, h, s, N.DS_SCATTER_KINEMATICAL, 1.0)
    return _out(F.real, scalar)


def _doyleturner(phase, h, s, voltage):
    volume = _volume(phase.structure.lattice)
    sites = _asymmetric_sites(phase.structure, phase.space_group)
    F = _family_F(sites, h, s, N.DS_SCATTER_DOYLETURNER, volume)
    # relativistic epilogue of structure_factor.py:164-172, on the device
    gamma_relcor = 1 + (2 * _E * 0.5 * voltage / _REST_MASS / (_C ** 2))
    v_mod = torch.abs(F) * gamma_relcor
    v_phase = torch.atan2(F.imag, F.real)
    v_g = torch.polar(v_mod, v_phase)
    pre = 2 * (_REST_MASS * _E / _H ** 2) * 1e-18
    return (pre * v_g).real, gamma_relcor, v_mod, v_phase, v_g


def get_doyleturner_structure_factor(phase, hkl, scattering_parameter, voltage, return_parameters=False):
    """Structure factor of the family hkl with Doyle-Turner scattering factors
    and the relativistic correction (diffsims/structure_factor/structure_factor.py:103-185).
    ``voltage`` in V.  With ``return_parameters`` also returns the dict
    ``gamma_relcor, v_mod, v_phase, v_g``."""
    h, s, scalar = _families(hkl, scattering_parameter)
    sf, gamma, v_mod, v_phase, v_g = _doyleturner(phase, h, s, voltage)
    if not return_parameters:
        return _out(sf, scalar)
    params = {"gamma_relcor": gamma, "v_mod": _out(v_mod, scalar), "v_phase": _out(v_phase, scalar),
              "v_g": _out(v_g, scalar)}
    return _out(sf, scalar), params


def get_refraction_corrected_wavelength(phase, voltage):
    """Refraction-corrected relativistic wavelength (Angstrom) for a voltage
    in V (diffsims/structure_factor/structure_factor.py:188-233): the mean
    inner potential is the Doyle-Turner v_mod of the 000 family."""
    temp1 = 1e9 * _H / np.sqrt(2 * _REST_MASS * _E)
    temp2 = _E * 0.5 * voltage / _REST_MASS / (_C ** 2)
    psi_hat = voltage * (1 + temp2)
    _, _, v_mod, _, _ = _doyleturner(phase, np.zeros((1, 3)), np.zeros(1), voltage)
    psi_hat += float(v_mod[0])
    return temp1 / np.sqrt(psi_hat)


def _atom_factor(atom, scattering_parameter, kind, volume):
    s = np.asarray(scattering_parameter, dtype=np.float64)
    scalar = s.ndim == 0
    s = s.reshape(-1)
    site = (_element_id(atom.element), np.zeros((1, 3)), float(getattr(atom, "occupancy", 1.0)), _biso(atom))
    F = _family_F([site], np.zeros((s.shape[0], 3)), s, kind, volume)
    return _out(F.real, scalar)


def get_kinematical_atomic_scattering_factor(atom, scattering_parameter):
    """Kinematical (X-ray) atomic scattering factor with occupancy and
    Debye-Waller factor (diffsims/structure_factor/atomic_scattering_factor.py:27-66).
    ``atom.element`` is a symbol or an atomic number."""
    return _atom_factor(atom, scattering_parameter, N.DS_SCATTER_KINEMATICAL, 1.0)


def get_doyleturner_atomic_scattering_factor(atom, scattering_parameter, unit_cell_volume):
    """Doyle-Turner atomic scattering factor with occupancy and Debye-Waller
    factor (diffsims/structure_factor/atomic_scattering_factor.py:69-124)."""
    return _atom_factor(atom, scattering_parameter, N.DS_SCATTER_DOYLETURNER, float(unit_cell_volume))


def _structure_factors_fp64(structure, hkl, g2, scattering_params):
    """Complex F = sum_j f_j(g) occ_j exp(2 pi i h.x_j) (no Debye-Waller term)
    of the given reflections: ds_structure_factors, FP64 form."""
    lib = N.load_library()
    dev = torch.device("cuda", torch.cuda.current_device())
    els, xyz, occ = sites_of(structure)
    atoms = PackedAtoms(els, xyz, occ, np.zeros(len(els)), scattering_params, dev)
    n = hkl.shape[0]
    h = torch.as_tensor(np.ascontiguousarray(hkl, dtype=np.float64)).to(dev)
    g = torch.as_tensor(np.ascontiguousarray(g2, dtype=np.float64)).to(dev)
    F = torch.empty((max(n, 1), 2), dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    N.check(lib.ds_structure_factors(atoms.cstruct(), None, N.ptr(h), N.ptr(g), n, N.DS_FORM_FP64, None, None,
                                     N.ptr(F), None, 0, N.ptr(status), N.stream_handle()), "structure factors")
    N.check_device_status(status, "structure factors")
    F = F[:n].cpu().numpy()
    return F[:, 0] + 1j * F[:, 1]


def calculate_structure_factor(phase, hkl, scattering_params="xtables"):
    """ReciprocalLatticeVector.calculate_structure_factor
    (diffsims/crystallography/reciprocal_lattice_vector.py:647-720) for the
    vectors ``hkl`` ((..., 3) integer Miller indices) of ``phase``: the
    vectors are grouped into sets of symmetry-equivalent indices under the
    phase's point group (``get_hkl_sets``, :766-820), the complex structure
    factor of each set's first vector is computed on the GPU (FP64; the
    formula of diffsims/utils/sim_utils.py:256-304 without Debye-Waller
    factors, as the reference calls it) and given to every vector of the
    set.  ``phase.structure`` must hold every atom of the cell (the
    reference's ``sanitise_phase``).  Returns complex values of shape
    ``hkl.shape[:-1]``."""
    h = np.asarray(hkl, dtype=np.float64)
    shape = h.shape[:-1]
    h = h.reshape(-1, 3)
    structure = phase.structure
    recip = reciprocal_basis(structure.lattice)
    reps, _, family = symmetry_families(np.rint(h).astype(np.int64), recip,
                                        point_group_rotations(getattr(phase, "space_group", None)),
                                        return_inverse=True)
    g = h[reps] @ recip
    F = _structure_factors_fp64(structure, h[reps], np.sum(g * g, axis=1), scattering_params)
    return F[family].reshape(shape)
