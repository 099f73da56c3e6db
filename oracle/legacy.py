"""FP64 CPU oracle for the legacy single-orientation path -- TEST INFRASTRUCTURE.

Restates ``DiffractionGenerator.calculate_ed_data``
(diffsims/generators/diffraction_generator.py:192-331) with
``get_points_in_sphere`` (diffsims/utils/sim_utils.py:436-474), reusing the
shape-factor and intensity restatements of ``oracle.kinematic``.  Only
tests, ``smoke()`` and ``bench.py`` may import it.

Third-party arithmetic restated here (absent from the build container):
* diffpy.structure 3.0.2 ``Lattice``: the standard Cartesian frame of a
  lattice has c along z and b in the yz-plane (a* along x); ``recbase`` is the
  inverse of the base; ``reciprocal()`` is the lattice whose base vectors are
  the rows of ``recbase`` transposed (a*, b*, c* in the same frame);
  ``cartesian(u) = u @ base``; ``dist(u, v)`` is the metric-tensor norm of
  ``u - v``.  Called at diffraction_generator.py:237-241 and
  sim_utils.py:458-471.
* transforms3d ``euler2mat(ai, aj, ak, axes="rzxz")``: rotating axes z, x', z''
  -- the active rotation ``Rz(ai) @ Rx(aj) @ Rz(ak)``.  Called at
  diffraction_generator.py:243-249.

Parity of the combination is pinned by fixtures from the reference's own
``calculate_ed_data`` run on these restatements (tests/golden/make_golden.py)
and by the reference's tests (diffsims/tests/generators/test_diffraction_generator.py:131-215).
The frame conventions themselves are the restatements above.
"""
from __future__ import annotations

import itertools
import math

import numpy as np

from . import kinematic as ok


def diffpy_stdbase(a, b, c, alpha, beta, gamma) -> np.ndarray:
    """Rows a, b, c in diffpy's standard frame: c || z, b in the yz-plane."""
    ca, cb, cg = np.cos(np.deg2rad([alpha, beta, gamma]))
    sa, sb, sg = np.sin(np.deg2rad([alpha, beta, gamma]))
    vunit = math.sqrt(1.0 + 2.0 * ca * cb * cg - ca * ca - cb * cb - cg * cg)
    ar = sa / (a * vunit)
    cgr = (ca * cb - cg) / (sa * sb)
    sgr = math.sqrt(1.0 - cgr * cgr)
    return np.array([[1.0 / ar, -cgr / sgr / ar, cb * a],
                     [0.0, b * sa, b * ca],
                     [0.0, 0.0, c]])


class DiffpyLattice:
    """The parts of diffpy's ``Lattice`` the legacy path reads."""

    def __init__(self, a=1.0, b=1.0, c=1.0, alpha=90.0, beta=90.0, gamma=90.0, base=None):
        if base is None:
            # parameters are kept as given (diffpy's setLatPar)
            self.a, self.b, self.c, self.alpha, self.beta, self.gamma = a, b, c, alpha, beta, gamma
            base = diffpy_stdbase(a, b, c, alpha, beta, gamma)
        base = np.asarray(base, dtype=np.float64)
        self.base = base
        if not hasattr(self, "a"):
            # parameters derived from the base vectors (diffpy's setLatBase)
            self.a, self.b, self.c = (float(np.linalg.norm(base[i])) for i in range(3))
            self.alpha = math.degrees(math.acos(np.dot(base[1], base[2]) / (self.b * self.c)))
            self.beta = math.degrees(math.acos(np.dot(base[0], base[2]) / (self.a * self.c)))
            self.gamma = math.degrees(math.acos(np.dot(base[0], base[1]) / (self.a * self.b)))
        self.stdbase = diffpy_stdbase(self.a, self.b, self.c, self.alpha, self.beta, self.gamma)
        self.recbase = np.linalg.inv(base)
        self.metrics = base @ base.T

    def abcABG(self):
        return (self.a, self.b, self.c, self.alpha, self.beta, self.gamma)

    def reciprocal(self):
        return DiffpyLattice(base=self.recbase.T)

    def cartesian(self, u):
        return np.dot(u, self.base)

    def dist(self, u, v):
        d = np.asarray(u, dtype=np.float64) - np.asarray(v, dtype=np.float64)
        return np.sqrt((d * np.dot(d, self.metrics)).sum(axis=-1))


def points_in_sphere(reciprocal_lattice, reciprocal_radius):
    """get_points_in_sphere (diffsims/utils/sim_utils.py:436-474): indices
    (float), Cartesian coordinates and |g| of the box points with |g| < r."""
    a, b, c = reciprocal_lattice.a, reciprocal_lattice.b, reciprocal_lattice.c
    hmax, kmax, lmax = (np.floor(reciprocal_radius / x) for x in (a, b, c))
    pts = np.asarray(list(itertools.product(np.arange(-hmax, hmax + 1), np.arange(-kmax, kmax + 1),
                                            np.arange(-lmax, lmax + 1))))
    inside = np.abs(reciprocal_lattice.dist(pts, [0, 0, 0])) < reciprocal_radius
    idx = pts[inside]
    return idx, reciprocal_lattice.cartesian(idx), reciprocal_lattice.dist(idx, [0, 0, 0])


def euler2mat_rzxz(ai, aj, ak) -> np.ndarray:
    """Rotating-axes z-x'-z'' Euler angles (radians) -> Rz(ai) Rx(aj) Rz(ak)."""
    def rz(t):
        c, s = math.cos(t), math.sin(t)
        return np.array([[c, -s, 0.0], [s, c, 0.0], [0.0, 0.0, 1.0]])

    c, s = math.cos(aj), math.sin(aj)
    rx = np.array([[1.0, 0.0, 0.0], [0.0, c, -s], [0.0, s, c]])
    return rz(ai) @ rx @ rz(ak)


SHAPES = {"linear": ok.sf_linear, "atanc": ok.sf_atanc, "sinc": ok.sf_sinc, "sin2c": ok.sf_sin2c,
          "lorentzian": ok.sf_lorentzian, "binary": ok.sf_binary}


def calculate_ed_data(lattice: DiffpyLattice, elements, xyz, occupancy, dw, voltage_kv, reciprocal_radius,
                      rotation=(0, 0, 0), max_excitation_error=1e-2, shape_factor_width=None,
                      shape_factor_model="lorentzian", precession_angle=0.0, approximate_precession=True,
                      minimum_intensity=1e-20, scattering_params="lobato", quad=False, **shape_kwargs):
    """diffsims/generators/diffraction_generator.py:192-331.  Returns
    (coordinates (N, 3), indices (N, 3) float, intensities (N,), excitation
    errors (N,)) in the reference's order.  ``dw``: per-atom B.  With
    ``quad`` the precession average is the reference's adaptive quadrature,
    else the tight quadrature of ``oracle.kinematic``."""
    k0 = 1.0 / ok.electron_wavelength(voltage_kv)
    idx, g, gsp = points_in_sphere(lattice.reciprocal(), reciprocal_radius)
    R = euler2mat_rzxz(*np.deg2rad(np.asarray(rotation, dtype=np.float64)))
    g = np.matmul(R, g.T).T
    r_spot = np.sqrt(np.sum(np.square(g[:, :2]), axis=1))
    z_spot = g[:, 2]
    s = -np.sqrt(k0 ** 2 - r_spot ** 2) + k0 - z_spot
    if precession_angle == 0:
        sel = np.abs(s) < max_excitation_error
    else:
        pz = k0 * np.cos(np.deg2rad(precession_angle))
        pt = k0 * np.sin(np.deg2rad(precession_angle))
        up = pz - np.sqrt(k0 ** 2 - (r_spot + pt) ** 2)
        do = pz - np.sqrt(k0 ** 2 - (r_spot - pt) ** 2)
        sel = (z_spot - max_excitation_error <= up) & (z_spot + max_excitation_error >= do)
    g, s, r_spot, idx, gsp = g[sel], s[sel], r_spot[sel], idx[sel], gsp[sel]
    w = max_excitation_error if shape_factor_width is None else shape_factor_width
    fn = SHAPES[shape_factor_model]
    if precession_angle == 0:
        shf = fn(s, w, **shape_kwargs)
    elif approximate_precession:
        shf = ok.sf_lorentzian_precession(s, w, r_spot, np.deg2rad(precession_angle))
    elif quad:
        shf = ok.sf_precession_integral(s, r_spot, np.deg2rad(precession_angle), fn, w, **shape_kwargs)
    else:
        shf = ok.sf_precession_integral_tight(s, r_spot, np.deg2rad(precession_angle), shape_factor_model, w,
                                              **shape_kwargs)
    inten = ok.kinematical_intensities(idx, gsp, elements, xyz, occupancy, dw, scattering_params, prefactor=shf)
    keep = inten > np.max(inten) * minimum_intensity
    return g[keep], idx[keep], inten[keep], s[keep]


def unique_families(hkls):
    """get_unique_families (diffsims/utils/sim_utils.py:101-136): classes of
    indices equal up to signs and order, in order of first appearance; each
    class is keyed by its lexicographically largest member, with its size."""
    classes = {}
    for h in hkls:
        key = tuple(sorted(np.abs(h)))
        classes.setdefault(key, []).append(list(h))
    return {tuple(sorted(v)[-1]): len(v) for v in classes.values()}


def calculate_profile_data(lattice: DiffpyLattice, elements, xyz, occupancy, dw, reciprocal_radius=1.0,
                           minimum_intensity=1e-3, scattering_params="lobato"):
    """DiffractionGenerator.calculate_profile_data
    (diffsims/generators/diffraction_generator.py:333-416) with
    get_intensities_params (diffsims/utils/sim_utils.py:513-556).  Returns
    (magnitudes, intensities scaled to 100, labels)."""
    rl = lattice.reciprocal()
    idx, _, dist = points_in_sphere(rl, reciprocal_radius)
    i_to_d = {tuple(i): d for i, d in zip(idx, dist)}
    fam = unique_families(idx.tolist())
    mult = np.fromiter(fam.values(), dtype=float)
    reps = np.array(list(fam))
    g = [i_to_d[tuple(u)] for u in reps]
    inten = ok.kinematical_intensities(reps, np.asarray(g), elements, xyz, occupancy, dw, scattering_params,
                                       prefactor=mult)
    labels_of = reps
    if (lattice.a == lattice.b and lattice.alpha == 90 and lattice.beta == 90 and lattice.gamma == 120):
        # the reference relabels with rows 0, 1, -(0 + 1), 2 of the family array
        labels_of = (reps[0], reps[1], -reps[0] - reps[1], reps[2])
    labels = ["".join(str(int(x)) for x in xs) for xs in labels_of]
    peaks = {}
    for lab, i, gg in zip(labels, inten, g):
        peaks[lab] = [i, gg]
    top = max(v[0] for v in peaks.values())
    x, y, hk = [], [], []
    for k, v in peaks.items():
        if v[0] / top * 100 > minimum_intensity and k != "000":
            x.append(v[1])
            y.append(v[0])
            hk.append(k)
    return x, np.asarray(y) / max(y) * 100, hk


def transformed_coordinates(coords, angle, center=(0, 0), mirrored=False):
    """In-plane turn of spot coordinates, the reference's operation order:
    theta = m atan2(y, x) + deg2rad(angle), r = |(x, y)|,
    (r cos theta + cx, r sin theta + cy).  Follows
    diffsims/sims/diffraction_simulation.py:199-215."""
    out = np.array(coords, dtype=np.float64, copy=True)
    x, y = out[:, 0], out[:, 1]
    theta = (-1 if mirrored else 1) * np.arctan2(y, x) + np.deg2rad(angle)
    rd = np.sqrt(x ** 2 + y ** 2)
    out[:, 0] = rd * np.cos(theta) + center[0]
    out[:, 1] = rd * np.sin(theta) + center[1]
    return out


def legacy_diffraction_pattern(calibrated_xy, intensities, shape=(512, 512), sigma=10, direct_beam_position=None,
                               in_plane_angle=0, mirrored=False):
    """DiffractionSimulation.get_diffraction_pattern: pixel positions, the
    in-frame spots truncated to int (last write wins), scipy
    ``gaussian_filter`` (via add_shot_and_point_spread without noise) and
    the division by the maximum; zeros when no spot is in the frame.
    Follows diffsims/sims/diffraction_simulation.py:296-354 and
    diffsims/pattern/detector_functions.py:64-80,109-141."""
    from scipy import ndimage as ndi
    if direct_beam_position is None:
        direct_beam_position = (shape[1] // 2, shape[0] // 2)
    c = transformed_coordinates(calibrated_xy, in_plane_angle, direct_beam_position, mirrored)
    inf = (c[:, 0] >= 0) & (c[:, 0] < shape[1]) & (c[:, 1] >= 0) & (c[:, 1] < shape[0])
    sc = c[inf].astype(int)
    si = np.asarray(intensities)[inf]
    pattern = np.zeros(shape)
    if si.shape[0] == 0:
        return pattern
    pattern[sc[:, 0], sc[:, 1]] = si
    pattern = ndi.gaussian_filter(pattern.T, sigma)
    return np.divide(pattern, np.max(pattern))


def legacy_mask(calibrated_xy, intensities, shape, radius=6.0, negative=True, radius_function=None,
                direct_beam_position=None, in_plane_angle=0, mirrored=False):
    """DiffractionSimulation.get_as_mask: a mask filled with ``negative``
    and discs (X - x)^2 + (Y - y)^2 < r^2 set to ``not negative``.  Follows
    diffsims/sims/diffraction_simulation.py:235-294 and
    diffsims/utils/mask_utils.py:24-28,64-116."""
    r = radius if radius_function is None else radius_function(np.asarray(intensities))
    if direct_beam_position is None:
        direct_beam_position = (shape[1] // 2, shape[0] // 2)
    c = transformed_coordinates(calibrated_xy, in_plane_angle, direct_beam_position, mirrored)
    mask = np.full(shape, negative, dtype=bool)
    X, Y = np.meshgrid(np.arange(shape[1]), np.arange(shape[0]))
    for (x, y), rr in zip(c[:, :2], r * np.ones(c.shape[0])):
        mask[(X - x) ** 2 + (Y - y) ** 2 < rr ** 2] = not negative
    return mask
