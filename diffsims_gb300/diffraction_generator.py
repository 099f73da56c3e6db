"""``DiffractionGenerator``: drop-in for the legacy single-structure generator
of diffsims/generators/diffraction_generator.py (``calculate_ed_data``),
running on the same CUDA kernels as ``SimulationGenerator``.

The legacy path differs from ``calculate_diffraction2d`` only in its inputs
and candidate set: a diffpy ``Structure`` in diffpy's standard frame (c along
z, b in the yz-plane), Euler angles in degrees in the rotating z-x-z
convention (transforms3d ``euler2mat(..., "rzxz")``, applied as ``R @ g``),
and the reciprocal-lattice points of ``get_points_in_sphere``
(diffsims/utils/sim_utils.py:436-474: the box of half-widths floor(r/|a*|),
... in itertools.product order, 000 included, |g| < r).  Excitation error,
selection, shape factors, intensities and the minimum-intensity mask are the
orientation kernel's.  Several Euler triples run as one launch.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native as N
from .crystal import Lattice, diffpy_base, lattice_params, sites_of
from .diffraction_simulation import DiffractionSimulation, ProfileSimulation
from .engine import PhaseTable, custom_shape_spots, simulate_phase
from .generator import SimulationGenerator
from .sim_utils import PackedAtoms, debye_waller_per_atom, get_electron_wavelength, get_kinematical_intensities


def structure_base(lattice) -> np.ndarray:
    """Direct base (rows a, b, c) of the legacy path's frame: a diffpy
    lattice's own ``base`` (which includes any ``baserot``), else diffpy's
    standard frame built from the cell parameters."""
    if not isinstance(lattice, Lattice) and hasattr(lattice, "base"):
        return np.asarray(lattice.base, dtype=np.float64).reshape(3, 3)
    return diffpy_base(*lattice_params(lattice))


def euler_rzxz_quaternions(euler_deg) -> np.ndarray:
    """Unit quaternions (w, x, y, z) of Rz(a) Rx(b) Rz(c) for Euler triples
    (degrees) in the rotating z-x-z convention: qz(a) * qx(b) * qz(c)."""
    e = np.deg2rad(np.atleast_2d(np.asarray(euler_deg, dtype=np.float64)).reshape(-1, 3)) / 2
    ca, sa = np.cos(e[:, 0]), np.sin(e[:, 0])
    cb, sb = np.cos(e[:, 1]), np.sin(e[:, 1])
    cc, sc = np.cos(e[:, 2]), np.sin(e[:, 2])
    # qz(a) * qx(b) = (ca cb, ca sb, sa sb, sa cb); then * qz(c)
    w1, x1, y1, z1 = ca * cb, ca * sb, sa * sb, sa * cb
    return np.stack([w1 * cc - z1 * sc, x1 * cc + y1 * sc, y1 * cc - x1 * sc, z1 * cc + w1 * sc], axis=1)


class DiffractionGenerator:
    """Electron diffraction spot patterns of one structure at given Euler
    angles.  Constructor arguments as diffsims/generators/diffraction_generator.py:155-191
    (``accelerating_voltage`` in kV, ``scattering_params``, ``precession_angle``
    in degrees, ``shape_factor_model`` by name or as the reference's model
    function, ``approximate_precession``, ``minimum_intensity``, shape-model
    keyword arguments); the same ``NotImplementedError`` for unknown names.
    ``shape_factor_model`` holds the model's name."""

    def __init__(self, accelerating_voltage, scattering_params="lobato", precession_angle=0,
                 shape_factor_model="lorentzian", approximate_precession=True, minimum_intensity=1e-20, **kwargs):
        self._gen = SimulationGenerator(accelerating_voltage, scattering_params, precession_angle,
                                        shape_factor_model, approximate_precession, minimum_intensity, **kwargs)
        self.wavelength = get_electron_wavelength(accelerating_voltage)
        self.precession_angle = self._gen.precession_angle
        self.approximate_precession = approximate_precession
        self.shape_factor_model = shape_factor_model
        self.minimum_intensity = minimum_intensity
        self.shape_factor_kwargs = kwargs
        self.scattering_params = scattering_params

    def calculate_ed_data(self, structure, reciprocal_radius, rotation=(0, 0, 0), with_direct_beam=True,
                          max_excitation_error=1e-2, shape_factor_width=None, debye_waller_factors={},
                          form="mixed"):
        """Spot pattern(s) of ``structure`` (diffraction_generator.py:192-331).

        ``rotation``: one Euler triple (degrees, rotating z-x-z) -> one
        ``DiffractionSimulation``; an (N, 3) array -> a list of N, from one
        launch.  ``form`` as ``SimulationGenerator.calculate_diffraction2d``.
        Fractional coordinates are used as given (the reference's re-basing
        at diffsims/utils/sim_utils.py:290-291 is the identity for lattices
        built from their parameters).  An orientation where nothing is
        selected gives an empty simulation (the reference raises).
        """
        if form not in ("mixed", "fp64"):
            raise ValueError("form must be 'mixed' or 'fp64'")
        N.load_library()
        dev = torch.device("cuda", torch.cuda.current_device())
        rot = np.asarray(rotation, dtype=np.float64)
        single = rot.ndim == 1
        rot = rot.reshape(-1, 3)
        recip = np.ascontiguousarray(np.linalg.inv(structure_base(structure.lattice)).T)
        els, xyz, occ = sites_of(structure)
        B = debye_waller_per_atom(els, debye_waller_factors)
        atoms = PackedAtoms(els, xyz, occ, B, self.scattering_params, dev)
        table = PhaseTable.sphere(recip, atoms, reciprocal_radius, form=form, device=dev)
        # the kernel writes R(q)^T g; the legacy path applies R(euler) g
        q = euler_rzxz_quaternions(rot)
        q[:, 1:] *= -1
        quats = torch.from_numpy(np.ascontiguousarray(q)).to(dev)
        settings = self._gen.settings(max_excitation_error, shape_factor_width, form)
        if self._gen._custom_shape is not None and settings.precession_mode != N.DS_PRECESSION_LORENTZIAN:
            # a shape-factor function of the caller's: evaluated on the host
            # between the selection and the finishing kernel
            spots = custom_shape_spots(table, quats, settings, reciprocal_radius, self._gen._custom_shape,
                                       self.shape_factor_kwargs)
        else:
            spots = simulate_phase(table, quats, settings, reciprocal_radius)
        off, idx, xyzi = spots.host(pinned=True)
        # one gather and one cast for all patterns; each simulation holds views
        hkl = table.hkl_host()[idx].astype(np.float64) if spots.total else np.zeros((0, 3))
        rec = xyzi.astype(np.float64)
        xyz, inten, o = rec[:, :3], rec[:, 3], off.tolist()
        make = DiffractionSimulation._from_arrays
        out = [make(xyz[a:b], hkl[a:b], inten[a:b], with_direct_beam) for a, b in zip(o[:-1], o[1:])]
        return out[0] if single else out

    def calculate_profile_data(self, structure, reciprocal_radius=1.0, minimum_intensity=1e-3,
                               debye_waller_factors={}):
        """1-D profile of ``structure`` (diffraction_generator.py:333-416):
        the sphere's reciprocal-lattice points (GPU enumeration) grouped into
        families of indices equal up to signs and order
        (get_unique_families, diffsims/utils/sim_utils.py:101-136; each keyed
        by its lexicographically largest member, weighted by its size), their
        intensities on the GPU, peaks labelled by hkl and scaled so the
        largest is 100; 000 and peaks at or below ``minimum_intensity`` are
        dropped.  A hexagonal cell (a == b, 90, 90, 120) is labelled as the
        reference does: with rows 0, 1, -(0 + 1) and 2 of the family array,
        which leaves four labels."""
        N.load_library()
        dev = torch.device("cuda", torch.cuda.current_device())
        lat = structure.lattice
        recip = np.ascontiguousarray(np.linalg.inv(structure_base(lat)).T)
        atoms = PackedAtoms(["H"], np.zeros((1, 3)), [1.0], [0.0], None, dev)  # enumeration only
        table = PhaseTable.sphere(recip, atoms, reciprocal_radius, device=dev)
        hkl = table.hkl_host()
        dist = np.sqrt(table.g2.cpu().numpy())
        classes = {}
        for h in hkl.tolist():
            classes.setdefault(tuple(sorted(abs(v) for v in h)), []).append(h)
        row_of = {tuple(h): r for r, h in enumerate(hkl.tolist())}
        reps = np.array([sorted(v)[-1] for v in classes.values()], dtype=np.float64).reshape(-1, 3)
        mult = np.array([len(v) for v in classes.values()], dtype=np.float64)
        g = dist[[row_of[tuple(int(x) for x in u)] for u in reps]]
        inten = get_kinematical_intensities(structure, reps, g, debye_waller_factors=debye_waller_factors,
                                            scattering_params=self.scattering_params, prefactor=mult)
        a, b, c, al, be, ga = lattice_params(lat)
        labels_of = reps
        if a == b and al == 90 and be == 90 and ga == 120:
            labels_of = (reps[0], reps[1], -reps[0] - reps[1], reps[2])
        labels = ["".join(str(int(x)) for x in xs) for xs in labels_of]
        peaks = {}
        for lab, i, gg in zip(labels, inten, g):
            peaks[lab] = [i, gg]
        top = max(v[0] for v in peaks.values())
        x, y, hkls = [], [], []
        for k, v in peaks.items():
            if v[0] / top * 100 > minimum_intensity and k != "000":
                x.append(v[1])
                y.append(v[0])
                hkls.append(k)
        return ProfileSimulation(x, np.asarray(y) / max(y) * 100, hkls)
