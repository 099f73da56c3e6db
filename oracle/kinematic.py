"""FP64 numpy restatement of diffsims' kinematical spot-pattern path.

TEST INFRASTRUCTURE ONLY (the checker): imported by tests/, by
``__graft_entry__.smoke()`` and by the CPU legs of ``bench.py``; never by the
``diffsims_gb300`` package.

Every function names the reference lines it follows (diffsims 0.7.x, paths
inside that project).  Geometry that the reference delegates to orix/diffpy
(which cannot be installed here) is restated from its published definition:

* lattice frame x || a, z || c* (orix ``Phase`` re-bases every structure to it;
  the reference's golden test relies on it, see
  diffsims/tests/generators/test_simulation_generator.py:311-313);
* Bunge Euler angles -> quaternion with the passive sign pattern of
  Rowenhorst et al., Modelling Simul. Mater. Sci. Eng. 23 (2015) 083501, eq. A.6
  (P = +1), as orix ``Rotation.from_euler`` does;
* ``~rotation * vector`` (diffsims/crystallography/_diffracting_vector.py:160)
  = R(q)^T g with R(q) the active (Hamilton) rotation matrix.
"""
from __future__ import annotations

import json
import math
import pathlib
import warnings
from dataclasses import dataclass, field

import numpy as np

# CODATA constants exactly as scipy.constants provides them (the reference
# imports them from there: diffsims/utils/sim_utils.py:25).
from scipy.constants import c as _C, e as _E, h as _H, m_e as _ME

_TABLES = json.loads(
    (pathlib.Path(__file__).resolve().parents[1] / "diffsims_gb300" / "data"
     / "scattering_params.json").read_text())


# --------------------------------------------------------------------------
# L1 physics: wavelength, scattering factors, structure factor
# --------------------------------------------------------------------------
def electron_wavelength(accelerating_voltage):
    """Relativistic electron wavelength in Angstrom for a voltage in kV.

    Follows diffsims/utils/sim_utils.py:57-79 (``get_electron_wavelength``).
    """
    if accelerating_voltage in (np.inf, "inf"):
        return 0
    E = accelerating_voltage * 1e3
    return _H / math.sqrt(2 * _ME * _E * E * (1 + (_E / (2 * _ME * _C * _C)) * E)) * 1e10


def element_symbol(atom_type_symbol: str) -> str:
    """Alphabetic head of a CIF atom type symbol.

    Follows diffsims/structure_factor/atomic_scattering_parameters.py:145-164.
    """
    i = 0
    while i < len(atom_type_symbol) and atom_type_symbol[i].isalpha() and atom_type_symbol[i].isascii():
        i += 1
    return atom_type_symbol[:i]


def scattering_coefficients(elements, scattering_params):
    """Per-atom (5, 2) coefficient array; unknown elements warn and give zeros.

    Follows diffsims/utils/sim_utils.py:139-162 and :198-219.
    """
    n = len(elements)
    coeffs = np.zeros((n, 5, 2))
    if scattering_params is None:
        return coeffs
    if scattering_params not in ("lobato", "xtables"):
        raise NotImplementedError(
            f"The scattering parameters `{scattering_params}` are not implemented.")
    table = _TABLES[scattering_params]
    for i, el in enumerate(elements):
        sym = element_symbol(el)
        if sym in table:
            coeffs[i] = np.asarray(table[sym])
        else:
            warnings.warn(f"Element {sym} from atom type symbol {el} not found in "
                          "scattering parameter library.")
    return coeffs


def atomic_scattering_factors(g_sq, coeffs, scattering_params):
    """f_j(g^2) for every (reflection, atom) pair.

    Follows diffsims/utils/sim_utils.py:227-253: Lobato
    f = sum_i a_i (2 + b_i g^2) / (1 + b_i g^2)^2; xtables f = sum_i a_i exp(-b_i g^2 / 4).
    """
    gb = np.outer(g_sq, coeffs[:, :, 1]).reshape(g_sq.shape + coeffs[:, :, 1].shape)
    if scattering_params == "lobato":
        f = (2 + gb) * (1 / np.square(1 + gb))
    elif scattering_params == "xtables":
        f = np.exp(-0.25 * gb)
    else:
        raise NotImplementedError(scattering_params)
    return np.sum(coeffs[:, :, 0] * f, axis=-1)


def structure_factor(hkl, g_spacing, elements, xyz, occupancy, dw, scattering_params="lobato"):
    """Complex kinematical structure factor F_hkl (float64).

    F = sum_j f_j(g) occ_j exp(2 pi i h.x_j - B_j g^2 / 4).  Follows
    diffsims/utils/sim_utils.py:256-304 with the fractional coordinates taken
    as given (the re-basing matrix at :290-291 is the identity in the
    x || a, z || c* frame).  ``dw`` is the per-atom B array (the reference maps
    element -> B through ``debye_waller_factors``, :220).
    """
    hkl = np.asarray(hkl, dtype=np.float64).reshape(-1, 3)
    g_sq = np.asarray(g_spacing, dtype=np.float64) ** 2
    coeffs = scattering_coefficients(elements, scattering_params)
    if scattering_params is not None:
        f = atomic_scattering_factors(g_sq, coeffs, scattering_params)
    else:
        f = np.ones((g_sq.shape[0], len(elements)))
    xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
    return np.sum(
        f * np.asarray(occupancy, dtype=np.float64)
        * np.exp(2j * np.pi * np.dot(hkl, xyz.T) - 0.25 * np.outer(g_sq, np.asarray(dw, np.float64))),
        axis=-1)


def kinematical_intensities(hkl, g_spacing, elements, xyz, occupancy, dw,
                            scattering_params="lobato", prefactor=1):
    """prefactor * |F|^2.  Follows diffsims/utils/sim_utils.py:307-354."""
    F = structure_factor(hkl, g_spacing, elements, xyz, occupancy, dw, scattering_params)
    return prefactor * (F * F.conjugate()).real


# --------------------------------------------------------------------------
# Shape factor models: diffsims/utils/shape_factor_models.py
# --------------------------------------------------------------------------
def sf_binary(s, w):
    """diffsims/utils/shape_factor_models.py:33-49 (returns the scalar 1)."""
    return 1


def sf_linear(s, w):
    """diffsims/utils/shape_factor_models.py:52-73."""
    sf = 1 - np.abs(s) / w
    if isinstance(s, np.ndarray):
        sf[sf < 0.0] = 0.0
    else:
        sf = max(sf, 0.0)
    return sf


def sf_sinc(s, w, minima_number=5):
    """diffsims/utils/shape_factor_models.py:76-101 (s = 0 gives 0, not 1)."""
    fac = np.pi * minima_number / w
    num = np.sin(fac * s)
    denom = fac * s
    return np.nan_to_num(np.abs(np.divide(num, denom, out=np.zeros_like(num), where=denom != 0)), nan=1)


def sf_sin2c(s, w, minima_number=5):
    """diffsims/utils/shape_factor_models.py:104-123."""
    return sf_sinc(s, w, minima_number) ** 2


def sf_atanc(s, w, minima_number=5):
    """diffsims/utils/shape_factor_models.py:126-151 (s = 0 gives 1)."""
    fac = np.pi * minima_number / np.abs(w)
    with np.errstate(invalid="ignore", divide="ignore"):
        return np.nan_to_num(np.arctan(fac * s) / (fac * s), nan=1)


def sf_lorentzian(s, w):
    """diffsims/utils/shape_factor_models.py:154-180."""
    sigma = np.pi / w
    return sigma / (np.pi * (sigma ** 2 * s ** 2 + 1)) * w


def sf_lorentzian_precession(s, w, r_spot, phi):
    """diffsims/utils/shape_factor_models.py:183-219 (phi in radians)."""
    sigma = np.pi / w
    u = sigma ** 2 * (r_spot ** 2 * phi ** 2 - s ** 2) + 1
    z = np.sqrt(u ** 2 + 4 * sigma ** 2 * s ** 2)
    return (sigma / np.pi) * np.sqrt(2 * (u + z) / z ** 2)


def sf_precession_integral(s, r_spot, phi, shape_function, w, **kwargs):
    """Rotation-averaged rel-rod factor by adaptive quadrature, per spot.

    Follows diffsims/utils/shape_factor_models.py:222-268 (scipy ``quad`` over
    theta in [0, 2 pi], default tolerances).
    """
    from scipy.integrate import quad
    out = np.zeros(np.shape(s))
    for i, (si, ri) in enumerate(zip(s, r_spot)):
        def integrand(theta, si=si, ri=ri):
            return shape_function(si + ri * phi * np.cos(theta), w, **kwargs)
        out[i] = (1 / (2 * np.pi)) * quad(integrand, 0, 2 * np.pi)[0]
    return out


def precession_breakpoint_step(model, w, minima_number=5):
    """Spacing in s of the points where the named model has a kink (linear:
    0 and +-w; sinc: its zeros at multiples of w/n), or the grid on which the
    smooth models are resolved (sin2c, atanc: w/2n; lorentzian: w/pi)."""
    aw = abs(w)
    return {"linear": aw, "sinc": aw / minima_number, "sin2c": aw / (2 * minima_number),
            "atanc": aw / (2 * minima_number), "lorentzian": aw / np.pi}.get(model, 0.0)


def sf_precession_integral_tight(s, r_spot, phi, model, w, **kwargs):
    """The same rotation average as :func:`sf_precession_integral` to ~1e-12:
    (1/pi) int_0^pi f(s + r phi cos t) dt by adaptive quadrature with the
    model's kinks given as break points and tight tolerances.  The reference's
    default tolerances leave an absolute error of up to ~2e-9; this is the
    yardstick for the relative error of small rotation averages."""
    from scipy.integrate import quad
    fn = ALL_SHAPE_MODELS[model]
    h = precession_breakpoint_step(model, w, **kwargs)
    out = np.zeros(np.shape(s))
    for i, (si, ri) in enumerate(zip(np.atleast_1d(s), np.atleast_1d(r_spot))):
        a = ri * phi
        if model == "binary":
            out[i] = 1.0
            continue
        if not a > 0:
            out[i] = fn(np.array([si]), w, **kwargs)[0]
            continue
        pts = []
        if h > 0:
            ks = np.arange(np.ceil((si - a) / h), np.floor((si + a) / h) + 1)
            pts = sorted(set(np.arccos(np.clip((ks * h - si) / a, -1, 1)).tolist()) - {0.0, np.pi})

        def integrand(t, si=si, a=a):
            return fn(np.array([si + a * np.cos(t)]), w, **kwargs)[0]
        v = quad(integrand, 0, np.pi, points=pts or None, epsabs=1e-15, epsrel=1e-12, limit=1000)[0]
        out[i] = v / np.pi
    return out


SHAPE_MODELS = {
    "linear": sf_linear,
    "atanc": sf_atanc,
    "sinc": sf_sinc,
    "sin2c": sf_sin2c,
    "lorentzian": sf_lorentzian,
}
#: models accepted by name by the reference (simulation_generator.py:49-55);
#: ``binary`` is reachable only as a callable there.
ALL_SHAPE_MODELS = dict(SHAPE_MODELS, binary=sf_binary)


# --------------------------------------------------------------------------
# L2 crystallography: lattice frame, hkl enumeration, rotations
# --------------------------------------------------------------------------
def lattice_base(a, b, c, alpha, beta, gamma):
    """Direct base (rows a, b, c) in the frame x || a, z || c* (degrees in).

    This is the frame orix ``Phase`` imposes on every structure
    (x="a", z="c*"); b lies in the xy-plane.
    """
    al, be, ga = np.deg2rad([alpha, beta, gamma])
    ca, cb, cg, sg = np.cos(al), np.cos(be), np.cos(ga), np.sin(ga)
    cx = c * cb
    cy = c * (ca - cb * cg) / sg
    cz = math.sqrt(max(c * c - cx * cx - cy * cy, 0.0))
    return np.array([[a, 0.0, 0.0], [b * cg, b * sg, 0.0], [cx, cy, cz]])


def reciprocal_base(base):
    """Rows a*, b*, c* (no 2 pi): g = hkl @ reciprocal_base(base)."""
    return np.linalg.inv(base).T


def g_cartesian(hkl, rbase):
    """g = h a* + k b* + l c*, evaluated in a fixed operation order.

    The order (h*a* + k*b*) + l*c*, then (gx^2 + gy^2) + gz^2, is the one the
    CUDA enumeration kernel uses with round-to-nearest intrinsics, so the
    d-spacing filter agrees bit for bit.
    """
    hkl = np.asarray(hkl, dtype=np.float64)
    h, k, l = hkl[..., 0:1], hkl[..., 1:2], hkl[..., 2:3]
    return (h * rbase[0] + k * rbase[1]) + l * rbase[2]


def g_squared(g):
    return (g[..., 0] * g[..., 0] + g[..., 1] * g[..., 1]) + g[..., 2] * g[..., 2]


def highest_hkl(rbase, min_dspacing):
    """Per-axis box half-widths: first n with 1/|n e_i| <= d_min.

    Follows the rule at diffsims/crystallography/get_hkl.py:49-57 (orix
    ``_get_highest_hkl``, called at reciprocal_lattice_vector.py:1131-1133).
    """
    out = np.ones(3, dtype=np.int64)
    for i in range(3):
        hkl = np.zeros(3)
        d = min_dspacing + 1
        while d > min_dspacing:
            hkl[i] += 1
            d = 1 / math.sqrt(g_squared(g_cartesian(hkl, rbase)))
        out[i] = int(hkl[i])
    return out


def enumerate_hkl(rbase, min_dspacing, n_zero=0):
    """Ordered hkl set of ``from_min_dspacing`` plus ``n_zero`` trailing 000 rows.

    Follows diffsims/crystallography/reciprocal_lattice_vector.py:1131-1141:
    box [H..-H]x[K..-K]x[L..-L] without 000, keep d = 1/|g| >= d_min, unique
    vectors in descending (h, k, l) order (orix ``Vector3d.unique`` sorts the
    Cartesian rows and reverses them; in the x || a, z || c* frame that is
    descending lexicographic hkl), then 000 appended when
    ``include_zero_vector``; generators/simulation_generator.py:351-353 appends
    a second 000 when the direct beam is on (``n_zero=2``).
    """
    H, K, L = highest_hkl(rbase, min_dspacing)
    hh, kk, ll = np.meshgrid(np.arange(H, -H - 1, -1), np.arange(K, -K - 1, -1),
                             np.arange(L, -L - 1, -1), indexing="ij")
    hkl = np.stack([hh.ravel(), kk.ravel(), ll.ravel()], axis=1)
    hkl = hkl[~np.all(hkl == 0, axis=1)]
    d = 1.0 / np.sqrt(g_squared(g_cartesian(hkl, rbase)))
    hkl = hkl[d >= min_dspacing]
    if n_zero:
        hkl = np.vstack([hkl, np.zeros((n_zero, 3), dtype=hkl.dtype)])
    return hkl.astype(np.int64)


def euler_to_quaternion(euler, degrees=False):
    """Bunge (phi1, Phi, phi2) -> unit quaternion (w, x, y, z), w >= 0.

    Passive convention with P = +1 (Rowenhorst et al. 2015, eu2qu), as orix
    ``Rotation.from_euler(direction="lab2crystal")``.
    """
    e = np.atleast_2d(np.asarray(euler, dtype=np.float64))
    if degrees:
        e = np.deg2rad(e)
    p1, P, p2 = e[:, 0], e[:, 1], e[:, 2]
    sig = 0.5 * (p1 + p2)
    dlt = 0.5 * (p1 - p2)
    c, s = np.cos(P / 2), np.sin(P / 2)
    q = np.stack([c * np.cos(sig), -s * np.cos(dlt), -s * np.sin(dlt), -c * np.sin(sig)], axis=1)
    q[q[:, 0] < 0] *= -1
    return q


def quaternion_to_matrix(q):
    """Active rotation matrix of unit quaternions (w, x, y, z), shape (N, 3, 3)."""
    q = np.atleast_2d(np.asarray(q, dtype=np.float64))
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
        np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
        np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1),
    ], axis=1)


def random_quaternions(n, seed=0):
    """Uniform SO(3): normalised standard-normal 4-vectors, canonical w >= 0."""
    rng = np.random.default_rng(seed)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    q[q[:, 0] < 0] *= -1
    return q


# --------------------------------------------------------------------------
# L3: one phase, many orientations
# --------------------------------------------------------------------------
@dataclass
class Crystal:
    """Plain description of one phase (what the reference reads from
    ``phase.structure``): lattice parameters (Angstrom, degrees), per-atom
    element symbols, fractional xyz, occupancy and Debye-Waller B."""
    lattice: tuple
    elements: list
    xyz: np.ndarray
    occupancy: np.ndarray = None
    B: np.ndarray = None

    def __post_init__(self):
        self.xyz = np.asarray(self.xyz, dtype=np.float64).reshape(-1, 3)
        n = self.xyz.shape[0]
        self.occupancy = np.ones(n) if self.occupancy is None else np.asarray(self.occupancy, np.float64)
        self.B = np.zeros(n) if self.B is None else np.asarray(self.B, np.float64)

    @property
    def base(self):
        return lattice_base(*self.lattice)

    @property
    def rbase(self):
        return reciprocal_base(self.base)


@dataclass
class SimParams:
    """Constructor and call arguments of SimulationGenerator
    (generators/simulation_generator.py:74-146)."""
    accelerating_voltage: float = 200.0
    scattering_params: str = "lobato"
    precession_angle: float = 0.0
    shape_factor_model: str = "lorentzian"
    approximate_precession: bool = True
    minimum_intensity: float = 1e-20
    reciprocal_radius: float = 1.0
    with_direct_beam: bool = True
    max_excitation_error: float = 1e-2
    shape_factor_width: float = None
    shape_kwargs: dict = field(default_factory=dict)
    # approximate_precession=False: "reference" = the reference's adaptive
    # quadrature with its default tolerances, "tight" = break points + tight
    # tolerances (same integral, ~1e-12)
    precession_quadrature: str = "reference"


@dataclass
class Pattern:
    hkl: np.ndarray        # (n, 3) int
    xyz: np.ndarray        # (n, 3) beam-frame coordinates, 1/Angstrom
    intensity: np.ndarray  # (n,)
    excitation_error: np.ndarray = None
    index: np.ndarray = None  # position in the candidate (hkl table) order


def phase_table(crystal: Crystal, p: SimParams):
    """The per-phase candidate table: ordered hkl (with 0, 1 or 2 trailing
    000 rows), Cartesian g and |g|."""
    rb = crystal.rbase
    hkl = enumerate_hkl(rb, 1.0 / p.reciprocal_radius, n_zero=2 if p.with_direct_beam else 0)
    g = g_cartesian(hkl, rb)
    gs = np.sqrt(g_squared(g))
    return hkl, g, gs


def simulate_orientation(crystal, p, table, R, return_s=False):
    """One orientation, following generators/simulation_generator.py:211-241
    (intensities and the minimum-intensity mask) and :319-412 (rotation,
    excitation error, selection, shape factor).  ``R`` is the active rotation
    matrix; beam-frame vectors are R^T g."""
    hkl, g, gs = table
    rot = g @ R
    k0 = 1 / electron_wavelength(p.accelerating_voltage)
    r_spot = np.sqrt(np.sum(np.square(rot[:, :2]), axis=1))
    z = rot[:, 2]
    z_sphere = -np.sqrt(k0 ** 2 - r_spot ** 2) + k0
    s = z_sphere - z
    eps = p.max_excitation_error
    phi = np.deg2rad(abs(p.precession_angle))
    if phi == 0:
        sel = np.abs(s) < eps
    else:
        Pz, Pt = k0 * np.cos(phi), k0 * np.sin(phi)
        with np.errstate(invalid="ignore"):
            z_up = Pz - np.sqrt(k0 ** 2 - (r_spot + Pt) ** 2)
            z_do = Pz - np.sqrt(k0 ** 2 - (r_spot - Pt) ** 2)
            sel = (z - eps <= z_up) & (z + eps >= z_do)
    idx = np.nonzero(sel)[0]
    s_sel, r_sel = s[idx], r_spot[idx]
    w = eps if p.shape_factor_width is None else p.shape_factor_width
    model = p.shape_factor_model
    fn = ALL_SHAPE_MODELS[model] if isinstance(model, str) else model
    if phi == 0:
        sf = fn(s_sel, w, **p.shape_kwargs)
    elif p.approximate_precession:
        sf = sf_lorentzian_precession(s_sel, w, r_sel, phi)
    elif p.precession_quadrature == "tight" and isinstance(model, str):
        sf = sf_precession_integral_tight(s_sel, r_sel, phi, model, w, **p.shape_kwargs)
    else:
        sf = sf_precession_integral(s_sel, r_sel, phi, fn, w, **p.shape_kwargs)
    inten = kinematical_intensities(hkl[idx], gs[idx], crystal.elements, crystal.xyz,
                                    crystal.occupancy, crystal.B, p.scattering_params, prefactor=sf)
    inten = np.broadcast_to(np.asarray(inten, dtype=np.float64), idx.shape).copy()
    if idx.size:
        keep = inten > np.max(inten) * p.minimum_intensity
    else:
        keep = np.zeros(0, dtype=bool)
    idx = idx[keep]
    return Pattern(hkl=hkl[idx], xyz=rot[idx], intensity=inten[keep],
                   excitation_error=s[idx] if return_s else None, index=idx)


def simulate(crystal: Crystal, quaternions, p: SimParams, return_s=False):
    """All orientations of one phase: list of ``Pattern``."""
    table = phase_table(crystal, p)
    Rs = quaternion_to_matrix(quaternions)
    return [simulate_orientation(crystal, p, table, R, return_s) for R in Rs]


def excitation_errors(crystal, p, table, R):
    """Beam-frame vectors and excitation error of every candidate (diagnostics)."""
    hkl, g, gs = table
    rot = g @ R
    k0 = 1 / electron_wavelength(p.accelerating_voltage)
    r_spot = np.sqrt(np.sum(np.square(rot[:, :2]), axis=1))
    return rot, (-np.sqrt(k0 ** 2 - r_spot ** 2) + k0) - rot[:, 2]


# --------------------------------------------------------------------------
# L5: rasterisation (Simulation2D.get_diffraction_pattern)
# --------------------------------------------------------------------------
def transformed_pixel_coordinates(xyz, shape, calibration, in_plane_angle=0.0, mirrored=False,
                                  direct_beam_position=None, fast=True):
    """Spot centres in pixels: divide by the calibration, rotate/mirror in
    plane, shift to the centre.  Follows
    diffsims/simulations/simulation2d.py:261-285 and :407-421."""
    if direct_beam_position is None:
        direct_beam_position = (shape[1] // 2, shape[0] // 2) if fast else \
            ((shape[1] - 1) / 2, (shape[0] - 1) / 2)
    cx, cy = direct_beam_position
    data = np.asarray(xyz, dtype=np.float64) / calibration
    x, y = data[:, 0], data[:, 1]
    mf = -1 if mirrored else 1
    theta = mf * np.arctan2(y, x) + np.deg2rad(in_plane_angle)
    rd = np.sqrt(x ** 2 + y ** 2)
    out = data.copy()
    out[:, 0] = rd * np.cos(theta) + cx
    out[:, 1] = rd * np.sin(theta) + cy
    return out


def subpixel_gaussian(coords, intens, shape, sigma, clip_threshold=1.0):
    """Per-spot boxed Gaussian accumulation.  Follows
    diffsims/pattern/detector_functions.py:314-359."""
    out = np.zeros(shape)
    inds = np.transpose(np.indices(shape), (1, 2, 0))
    prefactor = 1 / (2 * np.pi * sigma ** 2)
    exp_prefactor = -1 / (2 * sigma ** 2)
    for i in range(intens.size):
        coord = coords[i][:2][::-1]
        it = intens[i]
        with np.errstate(invalid="ignore", divide="ignore"):
            radius = np.sqrt(np.log(clip_threshold / (prefactor * it)) / exp_prefactor)
        if np.isnan(radius):
            continue
        sl = (slice(max(0, int(np.ceil(coord[0] - radius))), min(shape[0], int(np.floor(coord[0] + radius + 1)))),
              slice(max(0, int(np.ceil(coord[1] - radius))), min(shape[1], int(np.floor(coord[1] + radius + 1)))))
        out[sl] += it * prefactor * np.exp(exp_prefactor * np.sum((inds[sl] - coord) ** 2, axis=-1))
    return out


def diffraction_pattern(xyz, intensity, shape, sigma=10, calibration=0.01, in_plane_angle=0.0,
                        mirrored=False, fast=True, normalize=True, clip_threshold=1.0,
                        direct_beam_position=None):
    """Detector image of one pattern.  Follows
    diffsims/simulations/simulation2d.py:357-442 and
    diffsims/pattern/detector_functions.py:251-311 (integer path: last write
    wins, then ``scipy.ndimage.gaussian_filter`` with its defaults)."""
    from scipy import ndimage as ndi
    t = transformed_pixel_coordinates(xyz, shape, calibration, in_plane_angle, mirrored,
                                      direct_beam_position, fast)
    inten = np.asarray(intensity, dtype=np.float64)
    in_frame = (t[:, 0] >= 0) & (t[:, 0] < shape[1]) & (t[:, 1] >= 0) & (t[:, 1] < shape[0])
    coords = t[in_frame]
    inten = inten[in_frame]
    if inten.shape[0] == 0:
        return np.zeros(shape)
    if fast:
        coords = coords.astype(int)
        out = np.zeros(shape)
        out[coords[:, 1], coords[:, 0]] = inten
        out = ndi.gaussian_filter(out, sigma)
    else:
        out = subpixel_gaussian(coords, inten, shape, sigma, clip_threshold)
    if normalize:
        out = np.divide(out, np.max(out))
    return out


# --------------------------------------------------------------------------
# polar templates
# --------------------------------------------------------------------------
def get_closest(array, values):
    """Index of the closest entry of the sorted ``array`` for each value, the
    upper one on ties.  Follows diffsims/simulations/simulation2d.py:767-781."""
    array = np.asarray(array)
    idxs = np.searchsorted(array, values, side="left")
    prev = (idxs == len(array)) | (np.fabs(values - array[np.maximum(idxs - 1, 0)])
                                   < np.fabs(values - array[np.minimum(idxs, len(array) - 1)]))
    idxs[prev] -= 1
    return idxs


def polar_flatten(patterns, radial_axes=None, azimuthal_axes=None):
    """(r, theta, intensity) templates padded to the largest pattern, from a
    list of (xyz (n, 3), intensity (n,)).  Follows
    diffsims/simulations/simulation2d.py:313-355 and
    diffsims/crystallography/_diffracting_vector.py:186-194."""
    max_n = max(len(i) for _, i in patterns)
    r_t = np.zeros((len(patterns), max_n))
    t_t = np.zeros((len(patterns), max_n))
    i_t = np.zeros((len(patterns), max_n))
    for k, (xyz, inten) in enumerate(patterns):
        xyz = np.asarray(xyz, dtype=np.float64).reshape(-1, 3)
        r = np.linalg.norm(xyz[:, :2], axis=1)
        t = np.arctan2(xyz[:, 1], xyz[:, 0])
        inten = np.asarray(inten, dtype=np.float64)
        if radial_axes is not None and azimuthal_axes is not None:
            r = get_closest(radial_axes, r)
            t = get_closest(azimuthal_axes, t)
            mask = (r < len(radial_axes) - 1) & (t < len(azimuthal_axes) - 1)
            r, t, inten = r[mask], t[mask], inten[mask]
        r_t[k, :len(r)] = r
        t_t[k, :len(r)] = t
        i_t[k, :len(inten)] = inten
    if radial_axes is not None and azimuthal_axes is not None:
        r_t = np.array(r_t, dtype=int)
        t_t = np.array(t_t, dtype=int)
    return r_t, t_t, i_t


# --------------------------------------------------------------------------
# 1-D profiles: SimulationGenerator.calculate_diffraction1d
# --------------------------------------------------------------------------
def unique_with_symmetry(hkl, rbase, rotations):
    """ReciprocalLatticeVector.unique(use_symmetry=True)
    (diffsims/crystallography/reciprocal_lattice_vector.py:1531-1548), with
    orix's point-group orbit of each vector taken as {h R} (R the rotation
    parts of the space group, acting on Miller indices) and orix's
    ``Vector3d.unique`` as order-preserving (the order from_min_dspacing
    keeps): per vector the orbit's Cartesian coordinates rounded to 6
    decimals, rows lexsorted (z, then y, then x), np.unique over the orbits,
    reversed.  Returns (rows, orbit sizes)."""
    hkl = np.asarray(hkl).reshape(-1, 3)
    n = hkl.shape[0]
    orbits = [hkl[i] @ np.asarray(rotations) for i in range(n)]  # (m, 3) per vector; row o = h R_o
    data = np.array([(o @ rbase).round(6) for o in orbits])
    data_sorted = np.zeros_like(data)
    for i in range(n):
        a = data[i]
        data_sorted[i] = a[np.lexsort(a.T)]
    _, idx = np.unique(data_sorted, return_index=True, axis=0)
    reps = idx[::-1]
    mult = np.array([len({tuple(r) for r in orbits[i].tolist()}) for i in reps], dtype=float)
    return reps, mult


def diffraction1d(crystal: "Crystal", rotations, scattering_params="lobato", minimum_intensity=1e-3):
    """calculate_diffraction1d (diffsims/generators/simulation_generator.py:261-317):
    from_min_dspacing at its default 0.7 Angstrom, families by
    ``unique_with_symmetry``, I = multiplicity |F|^2 scaled to 100, kept above
    ``minimum_intensity``; hkil for hexagonal cells.  Returns (|g|, I, indices)."""
    rb = crystal.rbase
    hkl = enumerate_hkl(rb, 0.7)
    g = np.sqrt(g_squared(g_cartesian(hkl, rb)))
    reps, mult = unique_with_symmetry(hkl, rb, rotations)
    hr = hkl[reps].astype(float)
    inten = kinematical_intensities(hr, g[reps], crystal.elements, crystal.xyz, crystal.occupancy, crystal.B,
                                    scattering_params, prefactor=mult)
    if np.allclose(crystal.lattice[3:], [90, 90, 120]):
        hr = np.column_stack([hr[:, 0], hr[:, 1], -(hr[:, 0] + hr[:, 1]), hr[:, 2]])
    inten = np.asarray(inten) / max(inten) * 100
    keep = inten > minimum_intensity
    return g[reps][keep], inten[keep], hr[keep]
