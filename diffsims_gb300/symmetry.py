"""Crystal symmetry used by the drop-in API (host logic on small integer
and coordinate arrays): space-group operations given as diffpy objects or
(R, t) pairs, orbits of fractional positions, the point group acting on
Miller indices, and families of symmetry-equivalent reflections.
"""
from __future__ import annotations

import numpy as np


def _space_group_operations(space_group):
    if space_group is None or (isinstance(space_group, (int, np.integer)) and int(space_group) == 1):
        return [(np.eye(3), np.zeros(3))]
    if isinstance(space_group, (int, np.integer)):
        raise NotImplementedError(
            f"space group {int(space_group)} given by number: pass its operations (a diffpy SpaceGroup, an object "
            "with iter_symops() / symop_list, or (R, t) pairs)")
    if hasattr(space_group, "iter_symops"):
        ops = list(space_group.iter_symops())
    elif hasattr(space_group, "symop_list"):
        ops = list(space_group.symop_list)
    else:
        ops = list(space_group)
    out = []
    for op in ops:
        R, t = (op.R, op.t) if hasattr(op, "R") else op
        out.append((np.asarray(R, dtype=np.float64).reshape(3, 3), np.asarray(t, dtype=np.float64).reshape(3)))
    return out


def expand_position(space_group, xyz, eps=1e-5):
    """Distinct images ``R xyz + t`` of a fractional position, reduced into
    [0, 1) (diffpy ``expandPosition(spacegroup, xyz)[0]``, called at
    diffsims/structure_factor/structure_factor.py:94,162)."""
    out = []
    xyz = np.asarray(xyz, dtype=np.float64)
    for R, t in _space_group_operations(space_group):
        p = R @ xyz + t
        p = p - np.floor(p)
        if any(np.all(np.abs((p - q) - np.rint(p - q)) < eps) for q in out):
            continue
        out.append(p)
    return np.array(out).reshape(-1, 3)


def point_group_rotations(space_group) -> np.ndarray:
    """Distinct rotation parts R (fractional basis, integer, improper ones
    included) of a space group's operations -- the point group that acts on
    Miller indices as h -> h R.  ``None`` or 1 gives the identity alone."""
    ops = _space_group_operations(space_group)
    return np.unique(np.array([np.rint(R).astype(np.int64) for R, _ in ops]), axis=0)


def symmetry_families(hkl, recip, rotations, return_inverse=False):
    """One representative per family of symmetry-equivalent indices, as
    ReciprocalLatticeVector.unique(use_symmetry=True)
    (diffsims/crystallography/reciprocal_lattice_vector.py:1531-1548): every
    vector's orbit {h R} in Cartesian coordinates rounded to 6 decimals, its
    rows sorted by (z, y, x), the distinct orbits in ascending order of those
    sorted rows, reversed; each family is represented by its first member in
    the input order.  Returns (rows of ``hkl``, multiplicities = orbit sizes).
    ``hkl`` (n, 3) integers, ``recip`` rows a*, b*, c*, ``rotations`` (m, 3, 3).
    With ``return_inverse`` also each row's family, as a position in the
    returned representatives."""
    hkl = np.asarray(hkl, dtype=np.int64).reshape(-1, 3)
    n = hkl.shape[0]
    if n == 0:
        empty = (np.zeros(0, dtype=np.int64), np.zeros(0))
        return empty + (np.zeros(0, dtype=np.int64),) if return_inverse else empty
    orbit = np.einsum("ni,oij->noj", hkl, np.asarray(rotations, dtype=np.int64))
    data = (orbit.astype(np.float64) @ np.asarray(recip, dtype=np.float64)).round(6)
    # per orbit: rows ordered by z, then y, then x (three stable sorts)
    for col in (0, 1, 2):
        order = np.argsort(data[:, :, col], axis=1, kind="stable")
        data = np.take_along_axis(data, order[:, :, None], axis=1)
        orbit = np.take_along_axis(orbit, order[:, :, None], axis=1)
    _, idx, inv = np.unique(data.reshape(n, -1), axis=0, return_index=True, return_inverse=True)
    reps = idx[::-1]
    mult = np.array([len({tuple(r) for r in orbit[i].tolist()}) for i in reps], dtype=np.float64)
    if return_inverse:
        return reps, mult, (len(idx) - 1) - np.asarray(inv).reshape(-1)
    return reps, mult
